"""Benchmark: particle-steps/s of the full SPH step on a 3D jittered lattice.

Workload (default): 4,096,000 particles (160^3 jittered cubic lattice, dx = 0.01, h = 1.3 dx,
v ~ N(0, 0.1), rho = 1000 (1 + U(-0.01, 0.01))), double precision, f64 fast arithmetic
(double-word pair terms within the 1e-10 f64 tolerance; `--mode native` for IEEE double).
A step = cell hash + stable radix sort + cell table + sorted gather + continuity pass (density
update) + momentum pass (velocity and position update).  The state (4M x 64 B = 256 MB) is larger than the 129 MB L2, so no flush is
needed between steps.

Output: one JSON line (rank 0).  `value` = particle-steps/s over the timed steps with the state
resident in HBM (CUDA events on the library's stream, max over ranks); `e2e` = the same metric
through the public C ABI with host buffers (pinned) copied in and out every step.

`--impl reference` times the CPU path on the host cores instead: the reference has no executable
particle path (its code generator returns text, prestige/src/codegen/simple_cpu.rs:3-22), so the
CPU arm is this project's oracle restatement of the method, OpenMP over all host threads.

Multi-GPU (torchrun): every rank runs an independent replica of the workload on its own GPU
(replicas only: the plain path is one spatial domain; see the design notes); value = all ranks'
particle-steps / the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic bytes per particle of the pair pass (f64): reads pos, vel, rho, m once (64 B),
# writes acc-equivalent state update and drho once (32 B).
PASS_BYTES_F64 = 96
PASS_BYTES_F32 = 48
# DRAM bytes per particle per pass launch measured by ncu on the 1,000,000-particle lattice
# (dram__bytes_read.sum + dram__bytes_write.sum of the pass kernel / N); see profiles/.
PASS_TRAFFIC_PER_PARTICLE = None

METRIC = "particle-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=4096000)
    p.add_argument("--precision", default="f64", choices=["f64", "f32"])
    p.add_argument("--mode", default="fast", choices=["fast", "native"])
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--cpu-sample-n", type=int, default=0, help="particles in the CPU-baseline sample (0: auto)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def dist_setup():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pgroup = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        pgroup = dist
    return rank, world, local, pgroup


def barrier(pgroup):
    if pgroup is not None:
        pgroup.barrier()


def allmax(pgroup, v):
    if pgroup is None:
        return v
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
    pgroup.all_reduce(t, op=pgroup.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_measure(w, steps, threads):
    """Oracle (CPU restatement of the method) on `w` for `steps` steps; particle-steps/s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import py_oracle
    py_oracle.num_threads(threads)
    f = w["fields"]
    f64 = w["config"]["precision"] == 1
    dt = np.float64 if f64 else np.float32
    st = py_oracle.SphState(np.asarray(f["pos"], dt), np.asarray(f["vel"], dt), np.asarray(f["rho"], dt),
                            np.asarray(f["mass"], dt), f64=f64)
    sec = py_oracle.sph_run(w["config"], st, steps)
    return w["n"] * steps / sec, sec


def workload(args, n=None):
    from prestige_gb300 import workloads
    return workloads.sph_lattice_3d(n=n or args.n, seed=2, precision=1 if args.precision == "f64" else 0,
                                    f64_mode=1 if args.mode == "fast" else 0)


def config_json(args, n):
    return {"workload": "sph_lattice_3d", "particles": n, "lattice": "jittered cubic, dx=0.01, jitter +-0.2dx",
            "h_over_dx": 1.3, "precision": args.precision, "arith": args.mode,
            "step": "hash+radix sort+cell table+sorted gather+continuity pass+momentum pass (symplectic Euler)",
            "l2": "state larger than L2 (no flush)", "parallelism": "replicas" if args.gpus > 1 else "single GPU"}


def run_reference(args, rank, world, pgroup):
    if rank != 0:
        return
    threads = cpu_threads()
    n = args.cpu_sample_n or args.n
    w = workload(args, n)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import py_oracle
    py_oracle.num_threads(threads)
    f = w["fields"]
    f64 = args.precision == "f64"
    dt = np.float64 if f64 else np.float32
    st = py_oracle.SphState(np.asarray(f["pos"], dt), np.asarray(f["vel"], dt), np.asarray(f["rho"], dt),
                            np.asarray(f["mass"], dt), f64=f64)
    if args.warmup:
        py_oracle.sph_run(w["config"], st, args.warmup)
    sec = py_oracle.sph_run(w["config"], st, args.steps)
    value = n * args.steps / sec
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.precision,
           "data": "synthetic", "config": config_json(args, n),
           "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                            "sample": "%d particles x %d steps (after %d warm-up steps), OpenMP over %d threads; "
                                      "the reference has no executable CPU particle path, so this is the "
                                      "project's C++ restatement of the method" % (n, args.steps, args.warmup,
                                                                                   threads)},
           "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_gpu(args, rank, world, local, pgroup):
    import torch

    from prestige_gb300 import ParticleSystem, make_config, workloads

    torch.cuda.set_device(local)
    w = workload(args)
    n = w["n"]
    s = ParticleSystem(make_config(**w["config"]), n)
    workloads.load_into(s, w)
    info = s.info()

    # ---- device-timed steps, state resident in HBM ----
    s.step(args.warmup)
    s.timing_enable(True)
    barrier(pgroup)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    s.step_async(args.steps)
    s.sync()
    t = s.timing_read()
    clk = clocks.stop()
    barrier(pgroup)
    s.timing_enable(False)
    region_ms = allmax(pgroup, t["region_ms"])
    ms_per_step = region_ms / args.steps
    value = world * n * args.steps / (region_ms * 1e-3)
    pass_ms = t["pass_ms"] / args.steps
    bpp = PASS_BYTES_F64 if args.precision == "f64" else PASS_BYTES_F32
    achieved = bpp * n / (pass_ms * 1e-3) / 1e9
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak, peak_src = float(json.load(f)["hbm_gbs"]), "measured"
    traffic = PASS_TRAFFIC_PER_PARTICLE * n if PASS_TRAFFIC_PER_PARTICLE else None

    # ---- end to end through the C ABI with pinned host buffers ----
    eb = 8 if args.precision == "f64" else 4
    npdt = np.float64 if eb == 8 else np.float32
    host = {}
    for k in ("pos", "vel", "rho", "mass"):
        arr = np.asarray(w["fields"][k], npdt).reshape(-1)
        pt = torch.empty(arr.size, dtype=torch.float64 if eb == 8 else torch.float32, pin_memory=True)
        pt.numpy()[:] = arr
        host[k] = pt
    outs = {k: torch.empty(host[k].numel(), dtype=host[k].dtype, pin_memory=True) for k in ("pos", "vel", "rho")}
    h2d = sum(v.numel() for v in host.values()) * eb
    d2h = sum(v.numel() for v in outs.values()) * eb
    f64 = eb == 8
    for _ in range(2):  # warm-up of the copy path
        for k, v in host.items():
            s.set_ptr(k, v.data_ptr(), v.numel(), f64)
        s.step(1)
        for k, v in outs.items():
            s.get_ptr(k, v.data_ptr(), v.numel(), f64)
    barrier(pgroup)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        for k, v in host.items():
            s.set_ptr(k, v.data_ptr(), v.numel(), f64)
        s.step(1)
        for k, v in outs.items():
            s.get_ptr(k, v.data_ptr(), v.numel(), f64)
    e2e_s = time.perf_counter() - t0
    barrier(pgroup)
    e2e_s = allmax(pgroup, e2e_s)
    e2e_value = world * n * args.e2e_steps / e2e_s
    nbr_mean = None

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            threads = cpu_threads()
            cn = args.cpu_sample_n or min(n, 1000000)
            cw = workload(args, cn)
            csteps = 2
            cval, csec = cpu_measure(cw, csteps, threads)
            cpu = {"value": cval, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                   "sample": "%d-particle lattice of the same construction x %d steps (%.1f s), OpenMP over %d "
                             "threads; the reference has no executable CPU path, so this is the project's C++ "
                             "restatement of the method" % (cn, csteps, csec, threads)}
        out = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.precision, "data": "synthetic (seeded jittered lattice)",
            "config": config_json(args, n),
            "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": args.e2e_steps},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "kernel": "sph_pass_kernel",
                         "peak_source": peak_src,
                         "bytes_per_particle": bpp},
            "stages_ms_per_step": {"neighbor_search": t["neighbor_ms"] / args.steps,
                                   "sorted_gather": t["gather_ms"] / args.steps, "pair_pass": pass_ms},
            "gpu_launches": int(t["launches"]),
            "clocks": clk,
            "cpu_baseline": cpu,
            "info": {"n_cells": info["n_cells"], "sort_passes": info["sort_passes"], "pass_grid": info["pass_grid"]},
        }
        print(json.dumps(out), flush=True)
    s.close()


def main():
    args = parse()
    rank, world, local, pgroup = dist_setup()
    try:
        if args.impl == "reference":
            run_reference(args, rank, world, pgroup)
        else:
            run_gpu(args, rank, world, local, pgroup)
    finally:
        if pgroup is not None:
            pgroup.destroy_process_group()


if __name__ == "__main__":
    main()
