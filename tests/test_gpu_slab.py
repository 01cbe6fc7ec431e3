"""The two-stage SPH step (pg_step_stage) and the slab decomposition on the GPU.

  * Stage 0 then stage 1 gives the bits of pg_step, in every arithmetic mode and on the
    overlapped 1M-particle schedule; stage 1 out of order is refused with PG_ESTATE.
  * Densities replaced between the stages are what the momentum pass uses: the result equals the
    oracle's stage 1 on the same replaced densities.
  * Two ranks on one GPU (separate processes and contexts, gloo for the host-staged halo
    exchange; no kernel of one rank waits on the other) run the slab decomposition of
    prestige_gb300/slab.py: in the IEEE mode the slabs reproduce the single-domain oracle run bit
    for bit, in the double-word mode within 1e-10.
  * Two DEM slabs (SlabDEM, cut along z, spheres crossing it with their contact history) reproduce
    the single-domain oracle run bit for bit, history included.
"""
import os
import pickle
import socket
import sys

import numpy as np
import pytest

import prestige_gb300._native as nat
from prestige_gb300 import ParticleSystem, make_config, workloads

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _handle(w, **over):
    cfg = dict(w["config"], **over)
    s = ParticleSystem(make_config(**cfg), w["n"])
    workloads.load_into(s, w)
    return s, cfg


@pytest.mark.parametrize("precision,mode", [(1, 0), (1, 1), (0, 0), (0, 1)])
def test_two_stages_equal_one_step(pg, precision, mode):
    w = workloads.sph_lattice_3d(n=5000, seed=6, precision=precision)
    a, _ = _handle(w, precision=precision, f64_mode=mode)
    b, _ = _handle(w, precision=precision, f64_mode=mode)
    for _ in range(3):
        a.step(1)
        b.step_stage(0)
        b.step_stage(1)
    for k in ("pos", "vel", "rho"):
        assert np.array_equal(a.get(k), b.get(k))


def test_two_stages_on_the_overlapped_schedule(pg):
    w = workloads.sph_lattice_3d(n=1000000, seed=13)
    a, _ = _handle(w, f64_mode=1)
    b, _ = _handle(w, f64_mode=1)
    assert b.info()["overlap_split"] > 0
    a.step(1)
    b.step_stage(0)
    b.step_stage(1)
    assert np.array_equal(a.get("pos"), b.get("pos")) and np.array_equal(a.get("rho"), b.get("rho"))


def test_replaced_densities_reach_the_momentum_pass(pg, oracle):
    w = workloads.dam_break_2d(dx=0.05)
    s, cfg = _handle(w, f64_mode=0)
    st = oracle.SphState(w["fields"]["pos"], w["fields"]["vel"], w["fields"]["rho"], w["fields"]["mass"])
    s.step_stage(0)
    oracle.sph_stage(cfg, st, 0)
    assert np.array_equal(s.get("rho"), st.rho)
    rho = st.rho * (1.0 + 1e-3 * np.sin(np.arange(w["n"])))  # the caller's densities
    s.set("rho", rho)
    st.cols[6][:] = rho
    s.step_stage(1)
    oracle.sph_stage(cfg, st, 1)
    assert np.array_equal(s.get("pos"), st.pos) and np.array_equal(s.get("vel"), st.vel)


def test_stage_order_is_enforced(pg):
    w = workloads.sph_lattice_3d(n=2000, seed=6)
    s, _ = _handle(w)
    with pytest.raises(nat.PgError) as e:
        s.step_stage(1)
    assert e.value.status == nat.PG_ESTATE
    s.step_stage(0)
    s.set("vel", w["fields"]["vel"])  # a field other than rho ends the pending stage
    with pytest.raises(nat.PgError) as e:
        s.step_stage(1)
    assert e.value.status == nat.PG_ESTATE
    with pytest.raises(nat.PgError) as e:
        s.step_stage(2)
    assert e.value.status == nat.PG_EINVAL


def _free_port():
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _case():
    w = workloads.dam_break_2d(dx=0.05)
    w["fields"]["vel"] = np.random.default_rng(3).normal(0.0, 0.5, size=w["fields"]["pos"].shape)
    w["fields"]["vel"][w["n_fluid"]:] = 0.0
    return w, 6


def _rank(rank, world, port, mode, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from prestige_gb300.slab import SlabSPH
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, nsteps = _case()
    cfg = dict(w["config"], f64_mode=mode)
    slab = SlabSPH(cfg, w["fields"], dist, axis=0)
    slab.run(nsteps)
    slab.close()
    pos, vel, rho = slab.gather()
    if rank == 0:
        with open(out, "wb") as f:
            pickle.dump((pos, vel, rho), f)
    dist.destroy_process_group()


@pytest.mark.parametrize("mode", [0, 1])
def test_two_slabs_on_the_gpu(pg, oracle, tmp_path, mode):
    import torch.multiprocessing as mp
    out = str(tmp_path / "slab.pkl")
    mp.start_processes(_rank, args=(2, _free_port(), mode, out), nprocs=2, join=True, start_method="spawn")
    with open(out, "rb") as f:
        pos, vel, rho = pickle.load(f)
    w, nsteps = _case()
    f = w["fields"]
    st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    oracle.sph_run(w["config"], st, nsteps)
    if mode == 0:
        assert np.array_equal(pos, st.pos) and np.array_equal(vel, st.vel) and np.array_equal(rho, st.rho)
    else:
        rel = lambda a, b: np.abs(a - b).max() / np.abs(b).max()
        assert rel(pos, st.pos) <= 1e-10 and rel(vel, st.vel) <= 1e-10 and rel(rho, st.rho) <= 1e-10


def _dem_case():
    w = workloads.dem_compressed_lattice(nside=(4, 4, 14), seed=2)
    w["config"]["dt"] = 2e-6
    w["fields"]["vel"][:, 2] = np.random.default_rng(5).normal(0.0, 40.0, size=w["n"])
    return w, 10


def _dem_rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from prestige_gb300.slab import SlabDEM
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, nsteps = _dem_case()
    slab = SlabDEM(w["config"], w["fields"], dist, axis=2)
    slab.run(nsteps)
    slab.close()
    res = slab.gather()
    if rank == 0:
        with open(out, "wb") as f:
            pickle.dump(res, f)
    dist.destroy_process_group()


def test_two_dem_slabs_on_the_gpu(pg, oracle, tmp_path):
    """Two DEM slabs (z cut, spheres crossing it with their contact history) on two GPU ranks
    reproduce the single-domain oracle run bit for bit, history included."""
    import torch.multiprocessing as mp
    out = str(tmp_path / "slabdem.pkl")
    mp.start_processes(_dem_rank, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    with open(out, "rb") as f:
        pos, vel, omega, hpid, hxi = pickle.load(f)
    w, nsteps = _dem_case()
    f = w["fields"]
    st = oracle.DemState(f["pos"], f["vel"], f["omega"], f["radius"], f["mass"], w["config"]["contact_capacity"])
    c, _ = oracle.dem_run(w["config"], st, nsteps)
    assert c > 0
    assert np.array_equal(pos, st.pos) and np.array_equal(vel, st.vel) and np.array_equal(omega, st.omega)
    assert np.array_equal(hpid.reshape(-1), st.hpid) and np.array_equal(hxi.reshape(-1), st.hxi)
