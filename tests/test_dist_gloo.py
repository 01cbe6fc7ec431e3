"""Multi-process paths of bench.py on the CPU, over gloo with two ranks.

The plain SPH path runs one independent replica per rank (no collective on the data path); the
only cross-rank operations are the barrier around the timed region and the max over ranks of
the timed duration.  These tests run those pieces, and the reference arm under
torch.distributed.run, with world size 2 on 127.0.0.1.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    # CPU ranks over gloo, also on a machine with GPUs
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import bench
    r, w, _, pg = bench.dist_setup()
    bench.barrier(pg)
    # rank r reports a duration of (r + 1) s for a replica of 1000 particle-steps
    slowest = bench.allmax(pg, float(r + 1))
    value = w * 1000 / slowest
    with open(os.path.join(out_dir, "rank%d.json" % r), "w") as f:
        json.dump({"rank": r, "world": w, "slowest": slowest, "value": value}, f)
    pg.destroy_process_group()


def test_replica_timing_is_max_over_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    res = [json.load(open(tmp_path / ("rank%d.json" % r))) for r in range(2)]
    for r in res:
        assert r["world"] == 2
        assert r["slowest"] == 2.0          # the max over ranks, seen by both ranks
        assert r["value"] == 2 * 1000 / 2.0  # all ranks' particle-steps over the slowest time
    del torch


def test_reference_arm_under_torchrun_prints_one_line_from_rank0():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--particles", "4096", "--steps", "2", "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="2", CUDA_VISIBLE_DEVICES="")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["metric"] == "particle-steps/s" and out["value"] > 0
    assert out["cpu_baseline"]["kind"] == "port"
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["e2e"]["d2h_bytes_per_step"] == 0
