"""Benchmark: particle-steps/s of the full SPH step on a 3D jittered lattice.

Workload (default): 4,096,000 particles (160^3 jittered cubic lattice, dx = 0.01, h = 1.3 dx,
v ~ N(0, 0.1), rho = 1000 (1 + U(-0.01, 0.01))), double precision, f64 fast arithmetic
(double-word pair terms within the 1e-10 f64 tolerance; `--mode native` for IEEE double).
A step = cell hash + stable radix sort + cell table + sorted gather + continuity pass (density
update) + momentum pass (velocity and position update).  The state (4M x 64 B = 256 MB) is larger than the 129 MB L2, so no flush is
needed between steps.

Output: one JSON line (rank 0).  `value` = particle-steps/s over the timed steps with the state
resident in HBM (CUDA events on the library's stream, max over ranks); `e2e` = the same metric
through the public C ABI with host buffers (pinned) copied in and out every step, pipelined
with the asynchronous field calls so the copies overlap the neighbouring steps.  `roofline`
describes the momentum pass, the step's longest kernel launch (the continuity pass, of about
the same total time, runs as two launches beside the neighbour lists).  Unless --no-extras, six more
sections on rank 0: `batched` (512 uneven 2D dam breaks in one handle vs looping the plain
handles), `adjoint` (backward / forward cost of the differentiable 3D workload), `dem`
(200,000 spheres: the settling run over its 5,000 steps, and a contact-dense compressed lattice),
`dam_break` (the 2D dam break at dx = 0.02 over its 2,000 steps), `drift` (the double-word
trajectory against the IEEE one over whole runs) and `sweep` (the
lattice at 256k, 1M and 4M particles in f64 and f32, double-word / fast and IEEE arithmetic).

`--impl reference` times the CPU path on the host cores instead: the reference has no executable
particle path (its code generator returns text, prestige/src/codegen/simple_cpu.rs:3-22), so the
CPU arm is this project's restatement of the method in its CPU timing build (cell-sorted arrays,
neighbour lists built once per step, OpenMP over all host threads).

Multi-GPU (torchrun): every rank runs an independent replica of the workload on its own GPU
(the 4M lattice fits one GPU, so the benchmark runs replicas; one system split across GPUs is
prestige_gb300/slab.py); value = all ranks' particle-steps / the slowest rank's time.  Unless
--no-extras, the line then also carries `batched_sharded`: the 512 dam breaks bin-packed over the
ranks by particle count (prestige_gb300/batch_shard.py, one batched handle per rank, nothing
exchanged while they step), all systems' particle-steps over the slowest rank's time.
"""
import argparse
import hashlib
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic bytes per particle of the momentum pass (the step's longest launch): reads
# pos, vel, rho', m once and writes pos, vel once.  3D f64: 64 + 48 = 112 B; f32: 56 B.
MOM_BYTES = {"f64": 112, "f32": 56}
# Algorithmic bytes per particle-step of the DEM contact pass with its fused integrator: reads
# pos, vel, omega (72 B), radius and mass (16 B); writes pos, vel, omega (72 B).
DEM_BYTES = 160
# The momentum pass's ncu figures (DRAM bytes per particle of one launch, FMA-pipe and issue
# activity) from a capture at 1,000,000 particles, f64 double-word mode, with the command that
# made it and a digest of the pass's sources at the time; the bench line scales the bytes by the
# particle count and says whether the digest matches the sources being run.
MOM_PROFILE = os.path.join(ROOT, "profiles", "momentum_pass_lattice1m.json")
PASS_SOURCES = ("prestige_gb300/csrc/pg_sph.cu", "prestige_gb300/csrc/pg_sph_pass.cuh",
                "prestige_gb300/csrc/pg_arith.cuh")

# Flops of the method (each +, -, *, / and sqrt of the oracle's f64 step one flop), counted by the
# oracle's flop census on the 110,592-particle lattice of the same construction (seed 2):
# per neighbour pair in each pass (position difference, r^2, spline, velocity term and, in the
# momentum pass, viscosity where the pair approaches) and per particle (Tait pressure, density
# update, velocity and position update).  tests/test_oracle_flops.py recomputes them.
FLOPS_SAMPLE_PARTICLES = 110592
FLOPS_PER_PAIR = {"continuity": 24.887, "momentum": 34.385}
FLOPS_PER_PARTICLE = 28

METRIC = "particle-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    # (--particles, not --n: torch.distributed.run would read --n as an abbreviation of its own options)
    p.add_argument("--particles", "--n", dest="n", type=int, default=4096000)
    p.add_argument("--precision", default="f64", choices=["f64", "f32"])
    p.add_argument("--mode", default="fast", choices=["fast", "native"])
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--cpu-sample-n", type=int, default=0, help="particles in the CPU-baseline sample (0: auto)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true", help="skip the batched, adjoint and DEM sections")
    p.add_argument("--no-autotune", action="store_true", help="keep the default block size and cell multiplier")
    p.add_argument("--block", type=int, default=0,
                   help="fixed block size of the list kernels instead of the autotuner's (with --cell-mult)")
    p.add_argument("--cell-mult", type=float, default=0.5, help="cell multiplier used with --block")
    p.add_argument("--mom-block", type=int, default=0, help="momentum-pass block size used with --block (0: --block)")
    p.add_argument("--ppw", type=int, default=32, help="particles per warp of the pair passes used with --block")
    p.add_argument("--section", default="all",
                   choices=["all", "batched", "adjoint", "dem", "dem_settling", "dem_dense", "dam_break", "sweep",
                            "drift"],
                   help="run only one extra section and print its JSON (for profiling)")
    p.add_argument("--dem-steps", type=int, default=5000, help="steps of the DEM settling section")
    p.add_argument("--adjoint-steps", type=int, default=500)
    p.add_argument("--adjoint-every", type=int, default=50)
    p.add_argument("--adjoint-modes", default="native,fast", help="comma list of native, fast")
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
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
            self.path = None

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


def cpu_model():
    """Host CPU model name (lscpu), for the CPU-baseline record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return None


def cpu_measure(w, steps, threads, warmup=1):
    """CPU timing build of the step (oracle/cpu_timing.cpp: cell-sorted arrays, neighbour lists
    built once per step, OpenMP over `threads`) on `w`: the faster of cell multipliers 1 and 1/2
    in a one-step trial, then `steps` timed steps.  Returns (particle-steps/s, seconds, multiplier)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import py_oracle
    py_oracle.timing_threads(threads)
    f = w["fields"]
    f64 = w["config"]["precision"] == 1
    dt = np.float64 if f64 else np.float32
    st = py_oracle.SphState(np.asarray(f["pos"], dt), np.asarray(f["vel"], dt), np.asarray(f["rho"], dt),
                            np.asarray(f["mass"], dt), f64=f64)
    trial = {}
    for mult in (1.0, 0.5):
        cfg = dict(w["config"], cell_multiplier=mult)
        py_oracle.sph_run_timing(cfg, st, warmup)
        trial[mult] = py_oracle.sph_run_timing(cfg, st, 1)
    mult = min(trial, key=trial.get)
    sec = py_oracle.sph_run_timing(dict(w["config"], cell_multiplier=mult), st, steps)
    return w["n"] * steps / sec, sec, mult


def cpu_record(value, threads, sample):
    return {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "cpu_model": cpu_model(), "nproc": os.cpu_count(),
            "build": "oracle/cpu_timing.cpp: g++ -O3 -ffp-contract=fast -funroll-loops -fopenmp (no -march: the "
                     "recipe builds on x86 and Arm hosts alike)",
            "sample": sample}


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
    value, sec, mult = cpu_measure(w, args.steps, threads, warmup=max(args.warmup, 1))
    sample = ("%d particles x %d steps (after %d warm-up steps and a one-step trial of cell multipliers 1 and "
              "1/2; %g used), OpenMP over %d threads; the reference has no executable CPU particle path, so "
              "this is the project's C++ restatement of the method" % (n, args.steps, max(args.warmup, 1), mult,
                                                                       threads))
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.precision,
           "data": "synthetic", "config": config_json(args, n),
           "cpu_baseline": cpu_record(value, threads, sample),
           "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def sources_digest(paths=PASS_SOURCES):
    """Digest of the code of the pass's sources: comments and blank space are left out, so that
    a comment edit does not mark the figures stale."""
    h = hashlib.sha256()
    for p in paths:
        with open(os.path.join(ROOT, p)) as f:
            text = f.read()
        text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
        text = re.sub(r"//[^\n]*", " ", text)
        h.update(" ".join(text.split()).encode())
    return h.hexdigest()[:16]


def momentum_profile():
    """The committed ncu figures of the momentum pass, and whether they were captured from the
    sources being run."""
    try:
        with open(MOM_PROFILE) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return None
    d["matches_sources"] = d.get("sources_digest") == sources_digest()
    return d


def _peak_hbm():
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bench_batched(steps=100, looped_steps=5, sync_steps=2):
    """512 independent 2D dam breaks: one batched handle (graph-replayed step) against looping
    the plain per-system handles over the same systems, (a) as the plain API is called, pg_step
    per system, and (b) enqueue-only with graph replay on 512 streams, synchronised once per
    step (the most favourable looping)."""
    import torch

    from prestige_gb300 import ParticleSystem, workloads
    systems = workloads.batched_dam_breaks()
    total = sum(w["n"] for w in systems)
    cfgs = [dict(w["config"], f64_mode=1) for w in systems]
    b = ParticleSystem.batch(cfgs, [w["n"] for w in systems])
    for k in ("pos", "vel", "rho", "mass"):
        b.set(k, np.concatenate([w["fields"][k] for w in systems]))
    # per-stage split of one batched step (eager steps with CUDA events at the stage boundaries)
    b.step(2)
    b.timing_enable(True)
    b.step_async(5)
    b.sync()
    tt = b.timing_read()
    b.timing_enable(False)
    stages = {"neighbor_search": tt["neighbor_ms"] / 5, "sorted_gather": tt["gather_ms"] / 5,
              "neighbor_lists": tt["list_ms"] / 5, "continuity_pass": tt["cont_ms"] / 5,
              "momentum_pass": (tt["pass_ms"] - tt["list_ms"] - tt["cont_ms"]) / 5,
              "step_eager": tt["region_ms"] / 5}
    info = b.info()
    b.enable_graph(True)
    b.step(3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.step(steps)
    tb = time.perf_counter() - t0
    b.close()
    hs = []
    for w, c in zip(systems, cfgs):
        h = ParticleSystem(c, w["n"])
        workloads.load_into(h, w)
        h.enable_graph(True)
        hs.append(h)
    for h in hs:
        h.step_async(2)
    for h in hs:
        h.sync()
    t0 = time.perf_counter()
    for _ in range(sync_steps):
        for h in hs:
            h.step(1)
    ts = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(looped_steps):
        for h in hs:
            h.step_async(1)
    for h in hs:
        h.sync()
    tl = time.perf_counter() - t0
    for h in hs:
        h.close()
    vb = total * steps / tb
    vl = total * looped_steps / tl
    vs = total * sync_steps / ts
    return {"workload": "512 independent 2D dam breaks, N_i log-uniform in [500, 50000] (seed 3), H_i in "
                        "[0.5, 2.0] m, per-system dx/h/c0/dt, f64 double-word mode",
            "systems": len(systems), "particles": total, "unit": "particle-steps/s",
            "batched_value": vb, "batched_ms_per_step": 1e3 * tb / steps,
            "looped_value": vs, "looped_ms_per_step": 1e3 * ts / sync_steps, "batched_over_looped": vb / vs,
            "looped_async_value": vl, "looped_async_ms_per_step": 1e3 * tl / looped_steps,
            "batched_over_looped_async": vb / vl,
            "stages_ms_per_step": stages,
            "stages_note": ("overlapped: neighbor_lists = lists of the first %d slots; continuity_pass = the "
                            "continuity pass over them beside the lists of the rest" % info["overlap_split"])
            if info.get("overlap_split") else "sequential stages",
            "timing": "host wall clock around graph-replayed steps, stream synchronised; stages from eager "
                      "steps with CUDA events"}


def bench_batched_sharded(rank, world, pgroup, steps=100):
    """The 512 dam breaks of `bench_batched` bin-packed over the ranks by particle count, one
    batched handle (graph-replayed step) per rank and no collective while they step: all systems'
    particle-steps over the slowest rank's time (the total work is fixed: strong scaling)."""
    import torch

    from prestige_gb300 import workloads
    from prestige_gb300.batch_shard import ShardedBatch
    systems = workloads.batched_dam_breaks()
    for w in systems:
        w["config"] = dict(w["config"], f64_mode=1)
    sb = ShardedBatch(systems, rank, world)
    try:
        sb.enable_graph(True)
        sb.step(3)
        torch.cuda.synchronize()
        barrier(pgroup)
        t0 = time.perf_counter()
        sb.step(steps)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        barrier(pgroup)
    finally:
        sb.close()
    tmax = allmax(pgroup, t)
    loads = sb.particles_per_rank()
    return {"workload": "the batched section's 512 dam breaks, f64 double-word mode", "ranks": world,
            "systems_per_rank": [len(x) for x in sb.packing], "particles_per_rank": loads,
            "unit": "particle-steps/s", "value": sum(loads) * steps / tmax, "ms_per_step": 1e3 * tmax / steps,
            "steps": steps, "scaling": "strong",
            "timing": "host wall clock around graph-replayed steps, stream synchronised, max over ranks"}


def bench_adjoint(nsteps=500, every=50, n=100000, modes=("native", "fast")):
    """Differentiable 3D SPH: forward with checkpoints, then the adjoint sweep (recompute +
    adjoint passes); cost of a backward step over a forward step."""
    import torch

    from prestige_gb300 import ParticleSystem, make_config, workloads
    w = workloads.differentiable_3d(n=n)
    out = {"workload": "100,000-particle jittered lattice, 8 Fourier velocity modes (0.05 m/s), loss = mean "
                       "squared distance to a seeded target, %d steps, checkpoints every %d" % (nsteps, every)}
    for mode, name in ((0, "native"), (1, "fast")):
        if name not in modes:
            continue
        s = ParticleSystem(make_config(**dict(w["config"], f64_mode=mode)), n)
        workloads.load_into(s, w)
        s.step(3)
        workloads.load_into(s, w)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.forward_checkpointed(nsteps, every)
        tf = time.perf_counter() - t0
        x = s.get("pos")
        g = 2.0 * (x - w["target"]) / n
        t0 = time.perf_counter()
        da, dB, _ = s.backward(g)
        tb = time.perf_counter() - t0
        s.close()
        out[name] = {"forward_ms_per_step": 1e3 * tf / nsteps, "backward_ms_per_step": 1e3 * tb / nsteps,
                     "backward_over_forward": tb / tf, "dL_dalpha": da, "dL_dB": dB}
    return out


def bench_dem(settle_steps=5000, sample_every=250, dense_steps=20, dense_warmup=3):
    """3D DEM, 200,000 spheres, f64, device-timed with CUDA events on the library's stream.
    (a) The settling workload (random sequential insertion, free fall) for its 5,000 steps: every
        `sample_every` steps one step is timed and its particle-particle contacts counted.
    (b) A contact-dense case of the same size: spheres on a compressed cubic lattice (50 x 50 x
        80, 2 % overlap, random velocities and spins) inside touching walls, so every contact path
        (normal, tangential history, Coulomb slip, torques, walls) runs in the timed steps."""
    return {"settling": bench_dem_settling(settle_steps, sample_every),
            "dense": bench_dem_dense(dense_steps, dense_warmup), "unit": "particle-steps/s",
            "timing": "CUDA events on the library's stream"}


def bench_dem_settling(settle_steps=5000, sample_every=250):
    from prestige_gb300 import ParticleSystem, workloads
    w = workloads.dem_settling(200000)
    s = ParticleSystem(w["config"], w["n"])
    workloads.load_into(s, w)
    s.enable_graph(True)
    samples = []
    graph_ms = []
    done = 0
    while done < settle_steps:
        t0 = time.perf_counter()
        s.step(sample_every - 1)  # graph-replayed, timed by the host clock (pg_step waits)
        graph_ms.append(1e3 * (time.perf_counter() - t0) / (sample_every - 1))
        s.timing_enable(True)  # the sampled step runs eagerly with stage events
        s.step_async(1)
        s.sync()
        t = s.timing_read()
        s.timing_enable(False)
        done += sample_every
        samples.append({"step": done, "contacts": s.dem_contacts(), "ms": t["region_ms"], "pass_ms": t["pass_ms"]})
    s.close()
    settle_ms = statistics.median([x["ms"] for x in samples])
    settling = {"workload": "200,000 spheres, r in [0.5, 1.0] mm, random sequential insertion in 0.1 x 0.1 x 0.3 m, "
                            "kn 1e5, e 0.9, mu 0.3, dt 1e-6, f64, %d steps" % settle_steps,
                "particles": w["n"], "steps": settle_steps, "timed": "one step in every %d" % sample_every,
                "ms_per_step_median": settle_ms, "value": w["n"] / (settle_ms * 1e-3),
                "graph_ms_per_step_median": statistics.median(graph_ms),
                "graph_value": w["n"] / (statistics.median(graph_ms) * 1e-3),
                "graph_timing": "host clock around %d graph-replayed steps between samples" % (sample_every - 1),
                "contacts_max": max(x["contacts"] for x in samples),
                "contacts_per_sample": [x["contacts"] for x in samples],
                "note": "the spheres fall together (g t^2 / 2 = 0.12 mm in 5 ms), so pair contacts only start "
                        "where the lowest spheres meet the floor"}
    return settling


def bench_dem_dense(dense_steps=20, dense_warmup=3):
    from prestige_gb300 import ParticleSystem, workloads
    d = workloads.dem_compressed_lattice(nside=(50, 50, 80))
    s = ParticleSystem(d["config"], d["n"])
    workloads.load_into(s, d)
    s.step(dense_warmup)
    s.timing_enable(True)
    s.step_async(dense_steps)
    s.sync()
    t = s.timing_read()
    s.timing_enable(False)
    contacts = s.dem_contacts()
    s.close()
    ms = t["region_ms"] / dense_steps
    pass_ms = t["pass_ms"] / dense_steps
    peak, peak_src = _peak_hbm()
    achieved = DEM_BYTES * d["n"] / (pass_ms * 1e-3) / 1e9
    dense = {"workload": "200,000 spheres (50 x 50 x 80) on a cubic lattice spaced 2r (1 - 0.02), r = 0.5 mm, "
                         "velocities N(0, 0.05) m/s, spins N(0, 50) rad/s, touching walls, f64",
             "particles": d["n"], "steps": dense_steps, "warmup": dense_warmup, "ms_per_step": ms,
             "value": d["n"] / (ms * 1e-3), "contacts_last_step": contacts,
             "stages_ms_per_step": {"neighbor_search": t["neighbor_ms"] / dense_steps,
                                    "sorted_gather": t["gather_ms"] / dense_steps, "contact_pass": pass_ms},
             "roofline": {"kernel": "dem_pass_kernel", "bound": "hbm", "bytes_per_particle": DEM_BYTES,
                          "achieved": achieved, "peak": peak, "peak_source": peak_src, "unit": "GB/s",
                          "frac": achieved / peak,
                          "binding_resource": "FP64 pipe (contact law and integrator in IEEE double)"}}
    return dense


def bench_dam(steps=2000):
    """The 2D dam break at dx = 0.02 (5,000 fluid + 1,518 wall particles), its 2,000 steps,
    graph-replayed, in both f64 modes: a small system, bound by launch latency rather than by
    any pipe (host clock around the run, stream synchronised)."""
    import torch

    from prestige_gb300 import ParticleSystem, make_config, workloads
    w = workloads.dam_break_2d(dx=0.02)
    out = {"workload": "2D dam break, dx = 0.02, 5,000 fluid + 1,518 wall particles, %d steps" % steps,
           "particles": w["n"], "steps": steps, "unit": "particle-steps/s",
           "timing": "host clock around the graph-replayed run"}
    for mode, name in ((1, "double_word"), (0, "ieee")):
        s = ParticleSystem(make_config(**dict(w["config"], f64_mode=mode)), w["n"])
        workloads.load_into(s, w)
        s.enable_graph(True)
        s.step(3)
        workloads.load_into(s, w)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.step(steps)
        sec = time.perf_counter() - t0
        front = float(s.get("pos")[:w["n_fluid"], 0].max())
        s.close()
        out[name] = {"ms_per_step": 1e3 * sec / steps, "value": w["n"] * steps / sec, "front_x_m": front}
    return out


def bench_drift(n=4096000, lattice_steps=100, lattice_every=10, dam_steps=2000, dam_every=100):
    """Trajectory drift of the double-word f64 mode: its trajectory against the IEEE f64 one (which
    reproduces the oracle bit for bit), without resetting the state, on the 4M lattice for 100
    steps and on the 2D dam break at dx = 0.02 for its 2,000 steps.  Deviation of a field =
    max_i |a_dw - a_ieee| / max_i |a_ieee|, maximum over the checkpoints."""
    from prestige_gb300 import ParticleSystem, make_config, workloads

    def run(w, nsteps, every):
        a = ParticleSystem(make_config(**dict(w["config"], precision=1, f64_mode=0)), w["n"])
        b = ParticleSystem(make_config(**dict(w["config"], precision=1, f64_mode=1)), w["n"])
        workloads.load_into(a, w)
        workloads.load_into(b, w)
        worst = {"pos": 0.0, "vel": 0.0, "rho": 0.0}
        for _ in range(every, nsteps + 1, every):
            a.step(every)
            b.step(every)
            for k in worst:
                ref = a.get(k)
                worst[k] = max(worst[k], float(np.abs(b.get(k) - ref).max() / np.abs(ref).max()))
        a.close()
        b.close()
        return worst

    lat = run(workloads.sph_lattice_3d(n=n, seed=2), lattice_steps, lattice_every)
    dam = run(workloads.dam_break_2d(dx=0.02), dam_steps, dam_every)
    return {"bound": max(max(lat.values()), max(dam.values())),
            "lattice": {"workload": "sph_lattice_3d, %d particles" % n, "steps": lattice_steps, "max_rel": lat},
            "dam_break": {"workload": "2D dam break, dx = 0.02 (5,000 fluid + 1,518 wall particles)",
                          "steps": dam_steps, "max_rel": dam},
            "against": "IEEE f64 mode (bit-exact with the oracle)",
            "norm": "max_i |a_dw - a_ieee| / max_i |a_ieee| per field, maximum over checkpoints every %d (lattice) "
                    "and %d (dam break) steps" % (lattice_every, dam_every)}


def bench_sweep(steps=100, warmup=3, sizes=(262144, 1000000, 4096000)):
    """The 3D lattice sweep over N and arithmetic: device-timed steps (CUDA events on the
    library's stream), cell multiplier 0.5, the block size (64, 128 or 256) that ran a 3-step
    trial fastest for the case, the arithmetic mode held fixed."""
    from prestige_gb300 import ParticleSystem, make_config, workloads
    cases = [("f64", 1, "double-word"), ("f64", 0, "IEEE"), ("f32", 1, "fast (FMA)"), ("f32", 0, "IEEE")]
    rows = []
    for n in sizes:
        for prec, mode, label in cases:
            w = workloads.sph_lattice_3d(n=n, seed=2, precision=1 if prec == "f64" else 0, f64_mode=mode)
            s = ParticleSystem(make_config(**w["config"]), w["n"])
            workloads.load_into(s, w)
            trials = {}
            for block in (64, 128, 256):  # the trial steps advance the state; warm-up follows
                s.set_tuning(block, 0.5, mode)
                s.step(1)
                s.timing_enable(True)
                s.step_async(3)
                s.sync()
                trials[block] = s.timing_read()["region_ms"]
                s.timing_enable(False)
            best = min(trials, key=trials.get)
            s.set_tuning(best, 0.5, mode)
            s.step(warmup)
            s.timing_enable(True)
            s.step_async(steps)
            s.sync()
            t = s.timing_read()
            s.timing_enable(False)
            s.close()
            ms = t["region_ms"] / steps
            rows.append({"particles": w["n"], "precision": prec, "arith": label, "block": best, "ms_per_step": ms,
                         "value": w["n"] / (ms * 1e-3)})
    return {"workload": "jittered cubic lattice, dx=0.01, jitter +-0.2dx, h=1.3dx, v ~ N(0, 0.1), "
                        "rho = 1000(1 + U(-0.01, 0.01)), seed 2", "steps": steps, "unit": "particle-steps/s",
            "tuning": "cell multiplier 0.5; block per case from a 3-step trial of 64, 128, 256", "results": rows}


def run_gpu(args, rank, world, local, pgroup):
    import torch

    from prestige_gb300 import ParticleSystem, make_config, workloads

    torch.cuda.set_device(local)
    if args.section != "all":
        if rank == 0:
            if args.section == "adjoint":
                res = bench_adjoint(args.adjoint_steps, args.adjoint_every, modes=args.adjoint_modes.split(","))
            else:
                res = {"batched": bench_batched, "dem": lambda: bench_dem(settle_steps=args.dem_steps),
                       "dem_settling": lambda: bench_dem_settling(args.dem_steps), "dem_dense": bench_dem_dense,
                       "dam_break": bench_dam, "sweep": bench_sweep, "drift": bench_drift}[args.section]()
            print(json.dumps({"section": args.section, args.section: res}), flush=True)
        return
    w = workload(args)
    n = w["n"]
    s = ParticleSystem(make_config(**w["config"]), n)
    workloads.load_into(s, w)
    tuning = None
    if args.block:
        s.set_tuning(args.block, args.cell_mult, 1 if args.mode == "fast" else 0)
        s.set_momentum_block(args.mom_block)
        s.set_particles_per_warp(args.ppw)
        tuning = {"block_size": args.block, "momentum_block": s.info()["momentum_block"],
                  "particles_per_warp": s.info()["particles_per_warp"], "cell_multiplier": args.cell_mult,
                  "fixed": True}
    elif not args.no_autotune:  # outside the timed region; the state is restored by the tuner
        tuning = s.autotune(trial_steps=16)  # 8-step trials picked block sizes 1-2 % off on some boxes
    info = s.info()
    from prestige_gb300._native import measure_fma_peaks
    fp64_peak, fp32_peak = measure_fma_peaks()  # ~10 ms of FMA chains, before the timed region

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
    K = args.steps
    list_ms = t["list_ms"] / K
    cont_ms = t["cont_ms"] / K
    mom_ms = (t["pass_ms"] - t["list_ms"] - t["cont_ms"]) / K
    bpp = MOM_BYTES[args.precision]
    achieved = bpp * n / (mom_ms * 1e-3) / 1e9
    peak, peak_src = _peak_hbm()
    prof = momentum_profile() if (args.precision, args.mode) == ("f64", "fast") else None
    traffic = prof["dram_bytes_per_particle"] * n if prof else None
    # neighbour pairs per particle from the lists of the last timed step (lengths only)
    pairs = float(s.pair_counts().mean())
    flops_pp = pairs * (FLOPS_PER_PAIR["continuity"] + FLOPS_PER_PAIR["momentum"]) + FLOPS_PER_PARTICLE
    flops_tf = flops_pp * n / (ms_per_step * 1e-3) / 1e12
    pass_tf = pairs * (FLOPS_PER_PAIR["continuity"] + FLOPS_PER_PAIR["momentum"]) * n / \
        ((cont_ms + mom_ms) * 1e-3) / 1e12

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
    # Every step uploads its inputs and downloads its result through the asynchronous C-ABI calls:
    # the inputs of step k+1 upload and the results of step k download while the steps run.
    def e2e_loop(steps):
        for _ in range(steps):
            for k, v in host.items():
                s.set_ptr_async(k, v.data_ptr(), v.numel(), f64)
            s.step_async(1)
            for k, v in outs.items():
                s.get_ptr_async(k, v.data_ptr(), v.numel(), f64)
        s.wait_io()

    e2e_loop(2)  # warm-up of the copy path
    barrier(pgroup)
    t0 = time.perf_counter()
    e2e_loop(args.e2e_steps)
    e2e_s = time.perf_counter() - t0
    barrier(pgroup)
    e2e_s = allmax(pgroup, e2e_s)
    e2e_value = world * n * args.e2e_steps / e2e_s
    s.close()
    sharded = bench_batched_sharded(rank, world, pgroup) if world > 1 and not args.no_extras else None

    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline:
            threads = cpu_threads()
            cn = args.cpu_sample_n or min(n, 1000000)
            cw = workload(args, cn)
            csteps = 3
            cval, csec, cmult = cpu_measure(cw, csteps, threads)
            cpu = cpu_record(cval, threads,
                             "%d-particle lattice of the same construction x %d steps (%.1f s, cell multiplier %g, "
                             "the faster of 1 and 1/2), OpenMP over %d threads; the reference has no executable "
                             "CPU path, so this is the project's C++ restatement of the method"
                             % (cn, csteps, csec, cmult, threads))
        out = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.precision, "data": "synthetic (seeded jittered lattice)",
            "config": config_json(args, n),
            "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": args.e2e_steps,
                    "method": "pinned host buffers; every step pg_set_field_async of pos, vel, rho, mass, "
                              "pg_step_async, pg_get_field_async of pos, vel, rho; host wall clock from the "
                              "first upload to pg_wait_io"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "sph_list_pass_kernel (momentum pass)", "peak_source": peak_src,
                         "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one momentum-pass "
                                            "launch at 1,000,000 particles (%.0f B per particle: mostly the per-entry "
                                            "cache and the lists), scaled by N; %s; captured with: %s"
                                            % (prof["dram_bytes_per_particle"],
                                               "captured from the sources being run" if prof["matches_sources"]
                                               else "STALE: the pass's sources changed since the capture",
                                               prof["command"])) if prof else None,
                         "bytes_per_particle": bpp,
                         "pipes_ncu": {k: prof[k] for k in ("fma_pipe_active_pct", "issue_active_pct",
                                                            "long_scoreboard_stalls_per_issue")} if prof else None,
                         "binding_resource": "FP32 issue (double-word f64 arithmetic) and the latency of the "
                                             "per-entry cache and record loads" if args.mode == "fast"
                         and args.precision == "f64" else ("FP64 pipe" if args.precision == "f64" else "FP32 issue")},
            "flops": {"per_particle_step": flops_pp, "pairs_per_particle": pairs,
                      "pairs_source": "mean length of the exact neighbour lists of the last timed step",
                      "per_pair": FLOPS_PER_PAIR, "per_particle": FLOPS_PER_PARTICLE,
                      "counted": "oracle flop census: each +, -, *, / and sqrt of the f64 step one flop; "
                                 "candidate tests of non-neighbours excluded",
                      "achieved_tflops": flops_tf, "pair_passes_tflops": pass_tf,
                      "fp64_fma_peak_tflops": fp64_peak, "fp32_fma_peak_tflops": fp32_peak,
                      "frac_fp64": flops_tf / fp64_peak, "frac_fp32": flops_tf / fp32_peak,
                      "peak_source": "measured in this run: pg_measure_fma_peaks (8 independent FMA chains "
                                     "per thread, 8 x 256 threads per SM)",
                      "note": "f64 flops of the method; the double-word mode computes them on the FP32 pipe "
                              "(several FP32 instructions per f64 flop), so frac_fp64 above 1 means the step runs "
                              "its f64 arithmetic faster than the FP64 pipe could"
                      if args.mode == "fast" and args.precision == "f64" else None},
            "stages_ms_per_step": {"neighbor_search": t["neighbor_ms"] / K, "sorted_gather": t["gather_ms"] / K,
                                   "neighbor_lists": list_ms, "continuity_pass": cont_ms, "momentum_pass": mom_ms},
            "stages_note": ("overlapped: neighbor_lists = lists of the first %d slots; continuity_pass = the "
                            "continuity pass over them beside the lists of the rest (second stream), then the "
                            "continuity pass over the rest" % info["overlap_split"]) if info.get("overlap_split")
            else "sequential stages",
            "gpu_launches": int(t["launches"]),
            "clocks": clk,
            "cpu_baseline": cpu,
            "info": {"n_cells": info["n_cells"], "sort_passes": info["sort_passes"], "pass_grid": info["pass_grid"],
                     "arith": info["arith"], "overlap_split": info.get("overlap_split", 0)},
            "tuning": tuning,
        }
        if sharded is not None:
            out["batched_sharded"] = sharded
        if not args.no_extras:
            out["batched"] = bench_batched()
            out["adjoint"] = bench_adjoint(args.adjoint_steps, args.adjoint_every,
                                           modes=args.adjoint_modes.split(","))
            out["dem"] = bench_dem()
            out["dam_break"] = bench_dam()
            out["drift"] = bench_drift(n)
            out["sweep"] = bench_sweep()
        print(json.dumps(out), flush=True)


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
