"""Slab decomposition with halo exchange (prestige_gb300/slab.py), on the CPU over gloo.

Each rank's slab runs on a stand-in handle that computes the two stages of a step with the oracle
(test infrastructure: the same split of the step as pg_step_stage), so these tests check the
host logic alone: cut points, halo selection, the densities sent back between the stages,
migration and the global-id ordering of the local systems.  The slabs together must reproduce
the single-domain oracle run bit for bit, with 2 and 3 ranks (the middle rank of 3 has two
neighbours), on the 2D dam break (walls, particles crossing the cuts) and on a 3D lattice.
The DEM slabs (SlabDEM, one oracle step per step) likewise, on a contact-dense lattice whose
spheres cross the z cuts with their tangential history: positions, velocities, spins and the
history (global ids) bit for bit.
"""
import os
import pickle
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class OracleHandle:
    """The calls SlabSPH makes on a handle, computed by the oracle (f64)."""

    def __init__(self, cfg, n):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import py_oracle
        self.o = py_oracle
        self.cfg = cfg
        self.n = n
        self.f = {}

    def set(self, name, values):
        self.f[name] = np.array(values, np.float64)

    def get(self, name):
        return self.f[name].copy()

    def step_stage(self, stage):
        st = self.o.SphState(self.f["pos"], self.f["vel"], self.f["rho"], self.f["mass"])
        self.o.sph_stage(self.cfg, st, stage)
        self.f["pos"], self.f["vel"], self.f["rho"] = st.pos, st.vel, st.rho.copy()

    def close(self):
        pass


def _case(name):
    sys.path.insert(0, ROOT)
    from prestige_gb300 import workloads
    if name == "dam2d":
        w = workloads.dam_break_2d(dx=0.05)
        # a disturbed column, so that particles cross the cuts within a few steps
        w["fields"]["vel"] = np.random.default_rng(3).normal(0.0, 0.5, size=w["fields"]["pos"].shape)
        w["fields"]["vel"][w["n_fluid"]:] = 0.0
        return w, 6
    return workloads.sph_lattice_3d(n=3000, seed=5), 4


def _worker(rank, world, port, name, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="1")
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from prestige_gb300.slab import SlabSPH
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, nsteps = _case(name)
    slab = SlabSPH(w["config"], w["fields"], dist, axis=0, make_handle=OracleHandle)
    counts = []
    for _ in range(nsteps):
        slab.step()
        counts.append(int(slab.gid.size))
    slab.close()
    pos, vel, rho = slab.gather()
    if rank == 0:
        with open(out, "wb") as f:
            pickle.dump({"pos": pos, "vel": vel, "rho": rho}, f)
    with open(out + ".r%d" % rank, "wb") as f:
        pickle.dump({"counts": counts, "gid": slab.gid}, f)
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("name", ["dam2d", "lattice3d"])
def test_slabs_reproduce_the_single_domain_run(oracle, tmp_path, world, name):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    out = str(tmp_path / "slab.pkl")
    mp.start_processes(_worker, args=(world, _free_port(), name, out), nprocs=world, join=True,
                       start_method="spawn")
    with open(out, "rb") as f:
        got = pickle.load(f)
    w, nsteps = _case(name)
    f = w["fields"]
    st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    oracle.sph_run(w["config"], st, nsteps)
    assert np.array_equal(got["pos"], st.pos)
    assert np.array_equal(got["vel"], st.vel)
    assert np.array_equal(got["rho"], st.rho)
    ranks = []
    for r in range(world):
        with open(out + ".r%d" % r, "rb") as fh:
            ranks.append(pickle.load(fh))
    assert all(min(x["counts"]) > 0 for x in ranks)  # every slab holds particles
    if name == "dam2d":  # particles crossed cuts: some rank's count changed during the run
        assert any(len(set(x["counts"])) > 1 for x in ranks)


# ---- DEM slabs -------------------------------------------------------------------------------
class OracleDemHandle:
    """The calls SlabDEM makes on a DEM handle, computed by the oracle (f64)."""

    def __init__(self, cfg, n):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import py_oracle
        self.o = py_oracle
        self.cfg = cfg
        self.n = n
        self.C = int(cfg.get("contact_capacity", 16))
        self.f = {}
        self.hp = np.full(n * self.C, 0xFFFFFFFF, np.uint32)
        self.hx = np.zeros(n * self.C * 3)

    def set(self, name, values):
        self.f[name] = np.array(values, np.float64)

    def get(self, name):
        return self.f[name].copy()

    def set_dem_history(self, pid, xi):
        self.hp = np.array(pid, np.uint32).reshape(-1)
        self.hx = np.array(xi, np.float64).reshape(-1)

    def dem_history(self):
        return self.hp.reshape(self.n, self.C).copy(), self.hx.reshape(self.n, self.C, 3).copy()

    def step(self, nsteps=1):
        st = self.o.DemState(self.f["pos"], self.f["vel"], self.f["omega"], self.f["radius"], self.f["mass"], self.C)
        st.hpid[:] = self.hp
        st.hxi[:] = self.hx
        c, _ = self.o.dem_run(self.cfg, st, nsteps)
        assert c >= 0, "contact slots overflowed"
        self.f["pos"], self.f["vel"], self.f["omega"] = st.pos, st.vel, st.omega
        self.hp, self.hx = st.hpid.copy(), st.hxi.copy()

    def close(self):
        pass


def _dem_case():
    """A contact-dense lattice whose spheres move fast along z (the cut axis), so that spheres
    cross the cuts with their contact history within a few steps."""
    sys.path.insert(0, ROOT)
    from prestige_gb300 import workloads
    w = workloads.dem_compressed_lattice(nside=(4, 4, 14), seed=2)
    w["config"]["dt"] = 2e-6
    w["fields"]["vel"][:, 2] = np.random.default_rng(5).normal(0.0, 40.0, size=w["n"])
    return w, 10


def _dem_worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="1")
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from prestige_gb300.slab import SlabDEM
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, nsteps = _dem_case()
    slab = SlabDEM(w["config"], w["fields"], dist, axis=2, make_handle=OracleDemHandle)
    owned = []
    for _ in range(nsteps):
        slab.step()
        owned.append(hash(slab.gid.tobytes()))
    slab.close()
    res = slab.gather()
    if rank == 0:
        with open(out, "wb") as f:
            pickle.dump(res, f)
    with open(out + ".r%d" % rank, "wb") as f:
        pickle.dump({"owned": owned}, f)
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_dem_slabs_reproduce_the_single_domain_run(oracle, tmp_path, world):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    out = str(tmp_path / "slabdem.pkl")
    mp.start_processes(_dem_worker, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    with open(out, "rb") as f:
        pos, vel, omega, hpid, hxi = pickle.load(f)
    w, nsteps = _dem_case()
    f = w["fields"]
    C = w["config"]["contact_capacity"]
    st = oracle.DemState(f["pos"], f["vel"], f["omega"], f["radius"], f["mass"], C)
    c, _ = oracle.dem_run(w["config"], st, nsteps)
    assert c > 0
    assert np.array_equal(pos, st.pos) and np.array_equal(vel, st.vel) and np.array_equal(omega, st.omega)
    assert np.array_equal(hpid.reshape(-1), st.hpid) and np.array_equal(hxi.reshape(-1), st.hxi)
    owned = []
    for r in range(world):
        with open(out + ".r%d" % r, "rb") as fh:
            owned.append(pickle.load(fh)["owned"])
    assert any(len(set(x)) > 1 for x in owned)  # spheres crossed cuts during the run


def test_dem_history_translation_round_trip():
    """SlabDEM's history helpers: global partner ids to local ids (partners absent from the local
    system dropped, the order of the rest kept, walls and the empty tail untouched) and back."""
    sys.path.insert(0, ROOT)
    from prestige_gb300.slab import NO_PARTNER, WALL_ID, SlabDEM

    class Bare(SlabDEM):
        def __init__(self, hpid, hxi):  # only the history state
            self.hpid = np.asarray(hpid, np.uint32)
            self.hxi = np.asarray(hxi, np.float64)

    E = NO_PARTNER
    hpid = [[7, 3, WALL_ID + 2, 9, E, E],
            [5, E, E, E, E, E],
            [E, E, E, E, E, E]]
    hxi = np.arange(3 * 6 * 3, dtype=np.float64).reshape(3, 6, 3) + 1.0
    s = Bare(hpid, hxi)
    gid_local = np.array([2, 3, 5, 7, 11])          # global id of each local particle
    g2l = np.full(12, -1, np.int64)
    g2l[gid_local] = np.arange(gid_local.size)
    lp, lx = s._history_to_local(g2l)
    # row 0: 7 -> 3, 3 -> 1, the wall kept, 9 (absent) dropped; its spring goes with it
    assert lp[0].tolist() == [3, 1, WALL_ID + 2, E, E, E]
    assert np.array_equal(lx[0, :3], hxi[0, :3]) and not lx[0, 3:].any()
    assert lp[1].tolist() == [2, E, E, E, E, E] and np.array_equal(lx[1, 0], hxi[1, 0])
    assert (lp[2] == E).all() and not lx[2].any()
    back = SlabDEM._history_to_global(lp, gid_local)
    assert back[0].tolist() == [7, 3, WALL_ID + 2, E, E, E]
    assert back[1].tolist() == [5, E, E, E, E, E]
