"""Batched systems shared out over ranks (prestige_gb300/batch_shard.py), on the CPU.

  * pack_systems puts every system on exactly one rank, in ascending order, the same way on every
    call, and keeps the largest rank within the list-scheduling bound (mean + largest system);
    on 512 log-uniform system sizes it is within 1 % of the mean.
  * Over gloo with 2 and 3 ranks, each rank's batched handle is a stand-in that steps every
    system with the oracle (test infrastructure), so these tests check the host logic alone: the
    rank's handle holds only its own systems, in their original order, and the gathered fields
    equal the oracle run of every system alone.
"""
import math
import os
import pickle
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from prestige_gb300.batch_shard import pack_systems  # noqa: E402


def test_every_system_on_one_rank():
    rng = np.random.default_rng(0)
    counts = rng.integers(0, 5000, size=97)
    for world in (1, 2, 3, 8):
        shares = pack_systems(counts, world)
        assert len(shares) == world
        flat = sorted(i for s in shares for i in s)
        assert flat == list(range(len(counts)))
        assert all(s == sorted(s) for s in shares)
        assert shares == pack_systems(counts, world)  # deterministic
        loads = [int(sum(counts[i] for i in s)) for s in shares]
        assert max(loads) <= sum(counts) / world + max(counts)


def test_balance_on_log_uniform_sizes():
    rng = np.random.default_rng(3)
    counts = np.round(np.exp(rng.uniform(math.log(500), math.log(50000), size=512))).astype(int)
    for world in (2, 4, 8):
        loads = [sum(int(counts[i]) for i in s) for s in pack_systems(counts, world)]
        assert max(loads) <= 1.01 * sum(loads) / world


def test_more_ranks_than_systems():
    shares = pack_systems([10, 20, 5], 5)
    assert sorted(i for s in shares for i in s) == [0, 1, 2]
    assert sum(1 for s in shares if not s) == 2
    assert shares[0] == [1]  # the largest system goes to rank 0


def test_bad_arguments():
    with pytest.raises(ValueError):
        pack_systems([1, 2], 0)
    with pytest.raises(ValueError):
        pack_systems([1, -2], 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class OracleBatch:
    """The calls ShardedBatch makes on a batched handle, every system stepped by the oracle."""

    def __init__(self, configs, counts):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import py_oracle
        self.o = py_oracle
        self.configs = list(configs)
        self.counts = [int(c) for c in counts]
        self.f = {}

    def set(self, name, values):
        self.f[name] = np.array(values, np.float64)

    def get(self, name):
        return self.f[name].copy()

    def step(self, nsteps=1):
        offs = np.concatenate([[0], np.cumsum(self.counts)])
        for c, a, b in zip(self.configs, offs[:-1], offs[1:]):
            st = self.o.SphState(self.f["pos"][a:b], self.f["vel"][a:b], self.f["rho"][a:b], self.f["mass"][a:b])
            self.o.sph_run(c, st, nsteps)
            self.f["pos"][a:b], self.f["vel"][a:b], self.f["rho"][a:b] = st.pos, st.vel, st.rho

    def close(self):
        pass


def _systems():
    from prestige_gb300 import workloads
    return workloads.batched_dam_breaks(n_systems=7, nmin=100, nmax=700, seed=8)


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="1")
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from prestige_gb300.batch_shard import ShardedBatch
    dist.init_process_group("gloo", rank=rank, world_size=world)
    made = []

    def make(configs, counts):
        made.append(list(counts))
        return OracleBatch(configs, counts)

    systems = _systems()
    sb = ShardedBatch(systems, rank, world, make_batch=make)
    sb.step(2)
    sb.step(1)
    got = sb.gather(dist)
    sb.close()
    with open(out + ".r%d" % rank, "wb") as f:
        pickle.dump({"made": made, "mine": sb.mine, "got": got}, f)
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_shards_reproduce_the_per_system_runs(oracle, tmp_path, world):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    out = str(tmp_path / "shard.pkl")
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    ranks = []
    for r in range(world):
        with open(out + ".r%d" % r, "rb") as f:
            ranks.append(pickle.load(f))
    systems = _systems()
    counts = [w["n"] for w in systems]
    shares = pack_systems(counts, world)
    for r, x in enumerate(ranks):
        assert x["mine"] == shares[r]
        assert x["made"] == ([[counts[i] for i in shares[r]]] if shares[r] else [])
    for w, (pos, vel, rho) in zip(systems, ranks[0]["got"]):
        f = w["fields"]
        st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
        oracle.sph_run(w["config"], st, 3)
        assert np.array_equal(pos, st.pos) and np.array_equal(vel, st.vel) and np.array_equal(rho, st.rho)
    for x in ranks[1:]:  # every rank gathers the same
        for a, b in zip(x["got"], ranks[0]["got"]):
            assert all(np.array_equal(u, v) for u, v in zip(a, b))
