"""Batched systems shared out over two ranks on the GPU (prestige_gb300/batch_shard.py).

Two ranks run as two processes on one GPU (separate contexts; the systems are independent, so no
kernel of one rank waits on the other and nothing is exchanged while they step; gloo gathers the
results on the host afterwards).  Each rank's batched handle holds only its own systems.
  * IEEE f64: every system equals the oracle run of that system alone, bit for bit.
  * Double-word f64: every system equals the same system stepped in the one batch of all
    systems, bit for bit (a system's result does not depend on the batch it is in).
"""
import os
import pickle
import socket
import sys

import numpy as np
import pytest

from prestige_gb300 import ParticleSystem, workloads
from prestige_gb300.batch_shard import pack_systems

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NSTEPS = 5


def _free_port():
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _systems(mode):
    systems = workloads.batched_dam_breaks(n_systems=9, nmin=200, nmax=2500, seed=11)
    for w in systems:
        w["config"] = dict(w["config"], f64_mode=mode)
    return systems


def _rank(rank, world, port, mode, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from prestige_gb300.batch_shard import ShardedBatch
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sb = ShardedBatch(_systems(mode), rank, world)
    sb.enable_graph(True)
    sb.step(2)
    sb.step(NSTEPS - 2)
    got = sb.gather(dist)
    n_local = sb.handle.n if sb.handle is not None else 0
    sb.close()
    with open(out + ".r%d" % rank, "wb") as f:
        pickle.dump({"got": got, "n_local": n_local, "mine": sb.mine}, f)
    dist.destroy_process_group()


def _run(tmp_path, mode):
    import torch.multiprocessing as mp
    out = str(tmp_path / "shard.pkl")
    mp.start_processes(_rank, args=(2, _free_port(), mode, out), nprocs=2, join=True, start_method="spawn")
    ranks = []
    for r in range(2):
        with open(out + ".r%d" % r, "rb") as f:
            ranks.append(pickle.load(f))
    return ranks


def test_two_ranks_ieee_match_the_oracle(pg, oracle, tmp_path):
    ranks = _run(tmp_path, 0)
    systems = _systems(0)
    counts = [w["n"] for w in systems]
    shares = pack_systems(counts, 2)
    for r in range(2):
        assert ranks[r]["mine"] == shares[r]
        assert ranks[r]["n_local"] == sum(counts[i] for i in shares[r])
    for w, (pos, vel, rho) in zip(systems, ranks[0]["got"]):
        f = w["fields"]
        st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
        oracle.sph_run(w["config"], st, NSTEPS)
        assert np.array_equal(pos, st.pos) and np.array_equal(vel, st.vel) and np.array_equal(rho, st.rho)


def test_two_ranks_double_word_match_the_whole_batch(pg, tmp_path):
    ranks = _run(tmp_path, 1)
    systems = _systems(1)
    b = ParticleSystem.batch([w["config"] for w in systems], [w["n"] for w in systems])
    for k in ("pos", "vel", "rho", "mass"):
        b.set(k, np.concatenate([w["fields"][k] for w in systems]))
    b.step(NSTEPS)
    pos, vel, rho = b.get("pos"), b.get("vel"), b.get("rho")
    b.close()
    o = 0
    for w, (p, v, r) in zip(systems, ranks[1]["got"]):
        n = w["n"]
        assert np.array_equal(p, pos[o:o + n]) and np.array_equal(v, vel[o:o + n]) and np.array_equal(r, rho[o:o + n])
        o += n
