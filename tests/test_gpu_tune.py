"""Autotuner of the SPH step (pg_autotune, pg_set_tuning) and its host-side cache.

The tuner may change the cell multiplier, the arithmetic mode and the block size, never the
method: after tuning, the state is the one before tuning, and steps stay within the f64
tolerance of the oracle (bit-exact when the IEEE mode and the original multiplier are kept).
"""
import json

import numpy as np
import pytest

from prestige_gb300 import ParticleSystem, make_config, workloads

pytestmark = pytest.mark.gpu

F64_TOL = 1e-10


def _system(w, **over):
    cfg = dict(w["config"])
    cfg.update(over)
    s = ParticleSystem(make_config(**cfg), w["n"])
    workloads.load_into(s, w)
    return s, cfg


def _rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


@pytest.mark.parametrize("graph", [False, True])
def test_autotune_restores_state_and_keeps_results(pg, oracle, graph):
    w = workloads.sph_lattice_3d(n=6000, seed=31)
    s, cfg = _system(w)
    if graph:
        s.enable_graph(True)
    before = s.get("pos"), s.get("vel"), s.get("rho")
    res = s.autotune(trial_steps=2)
    assert res["block_size"] in (64, 128, 256)
    assert res["cell_multiplier"] in (1.0, 0.5)
    assert res["f64_mode"] in (0, 1)
    assert res["ms_per_step"] > 0
    for a, b in zip((s.get("pos"), s.get("vel"), s.get("rho")), before):
        assert np.array_equal(a, b)
    info = s.info()
    assert info["graph"] == (1 if graph else 0)
    s.step(3)
    f = w["fields"]
    st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    oracle.sph_run(cfg, st, 3)
    assert _rel(s.get("pos"), st.pos) <= F64_TOL
    assert _rel(s.get("rho"), st.rho) <= F64_TOL
    s.close()


@pytest.mark.parametrize("block,mult", [(64, 0.5), (256, 1.0), (128, 0.5)])
def test_set_tuning_ieee_is_bit_exact(pg, oracle, block, mult):
    """IEEE mode with any block size and multiplier reproduces the oracle run with that multiplier."""
    w = workloads.sph_lattice_3d(n=4000, seed=32)
    s, cfg = _system(w)
    s.set_tuning(block, mult, 0)
    s.step(2)
    cfg = dict(cfg, cell_multiplier=mult)
    f = w["fields"]
    st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    oracle.sph_run(cfg, st, 2)
    assert np.array_equal(s.get("pos"), st.pos)
    assert np.array_equal(s.get("rho"), st.rho)
    s.close()


def test_autotune_cache_round_trip(pg, tmp_path):
    w = workloads.sph_lattice_3d(n=3000, seed=33)
    cache = str(tmp_path / "tuning.json")
    s, _ = _system(w)
    first = s.autotune(trial_steps=1, cache=cache)
    assert first["cached"] is False
    table = json.load(open(cache))
    assert s.tuning_key() in table
    s2, _ = _system(w)
    second = s2.autotune(trial_steps=1, cache=cache)
    assert second["cached"] is True
    assert second["block_size"] == first["block_size"]
    assert first["momentum_block"] in (64, 128, 256)
    assert s2.info()["momentum_block"] == first["momentum_block"]
    assert s2.info()["block_size"] == first["block_size"]
    assert s2.info()["pass_grid"] > 0
    s.close()
    s2.close()


def test_autotune_rejects_dem(pg):
    w = workloads.dem_settling(n=500)
    s = ParticleSystem(w["config"], w["n"])
    with pytest.raises(Exception):
        s.autotune(trial_steps=1)
    s.close()


@pytest.mark.parametrize("graph", [False, True])
def test_momentum_block_ieee_is_bit_exact(pg, oracle, graph):
    """The momentum pass's own block size changes the schedule only: IEEE mode stays bit-exact
    with the oracle for every momentum block, eager and from a graph."""
    w = workloads.sph_lattice_3d(n=4000, seed=34)
    s, cfg = _system(w)
    s.set_tuning(64, 1.0, 0)
    if graph:
        s.enable_graph(True)
    for mb in (256, 128, 0):
        s.set_momentum_block(mb)
        info = s.info()
        assert info["momentum_block"] == (mb or 64) and info["block_size"] == 64
        assert info["graph"] == (1 if graph else 0)
    s.set_momentum_block(256)
    s.step(2)
    f = w["fields"]
    st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    oracle.sph_run(dict(cfg, cell_multiplier=1.0), st, 2)
    assert np.array_equal(s.get("pos"), st.pos)
    assert np.array_equal(s.get("rho"), st.rho)
    s.set_tuning(128, 1.0, 0)  # a new tuning resets the momentum block to the common one
    assert s.info()["momentum_block"] == 128
    s.close()


def test_momentum_block_errors(pg):
    from prestige_gb300 import _native as nat
    w = workloads.sph_lattice_3d(n=500, seed=35)
    s, _ = _system(w)
    for bad in (-32, 16, 48, 2048):
        with pytest.raises(nat.PgError):
            s.set_momentum_block(bad)
    s.close()
    d = workloads.dem_settling(n=500)
    s = ParticleSystem(d["config"], d["n"])
    with pytest.raises(nat.PgError):
        s.set_momentum_block(128)
    s.close()


PPW_CASES = [
    ("lattice3d", lambda: workloads.sph_lattice_3d(n=4096, seed=2), 1),
    ("lattice3d_half", lambda: workloads.sph_lattice_3d(n=3000, seed=9, cell_multiplier=0.5), 1),
    ("dam2d", lambda: workloads.dam_break_2d(dx=0.05), 1),
    ("lattice3d_f32", lambda: workloads.sph_lattice_3d(n=4096, seed=2, precision=0), 0),
]


@pytest.mark.parametrize("ppw", [16, 8])
@pytest.mark.parametrize("name,make,f64", PPW_CASES)
def test_particles_per_warp_steps_within_tolerance(pg, oracle, ppw, name, make, f64):
    """Two or four threads per particle in the tolerance-based modes: each step (from the
    oracle's state) within the mode's bound, eager and graph-replayed (the same bits)."""
    w = make()
    s, cfg = _system(w, f64_mode=1)
    s.set_particles_per_warp(ppw)
    assert s.info()["particles_per_warp"] == ppw
    g, _ = _system(w, f64_mode=1)
    g.set_particles_per_warp(ppw)
    g.enable_graph(True)
    tol = F64_TOL if f64 else 1e-4
    dt = np.float64 if f64 else np.float32
    f = w["fields"]
    st = oracle.SphState(np.asarray(f["pos"], dt), np.asarray(f["vel"], dt), np.asarray(f["rho"], dt),
                         np.asarray(f["mass"], dt), f64=bool(f64))
    for _ in range(3):
        s.step(1)
        g.step(1)
        oracle.sph_run(cfg, st, 1)
        assert _rel(s.get("pos"), st.pos) <= tol
        assert np.abs(s.get("vel") - st.vel).max() <= tol * max(np.abs(st.vel).max(), cfg["dt"] * 1e3)
        assert _rel(s.get("rho"), st.rho) <= tol
        assert np.array_equal(g.get("pos"), s.get("pos")) and np.array_equal(g.get("rho"), s.get("rho"))
        for k in ("pos", "vel", "rho"):
            s.set(k, getattr(st, k))
            g.set(k, getattr(st, k))
    s.close()
    g.close()


def test_particles_per_warp_with_overflowed_lists(pg, oracle):
    """Lists shorter than the neighbourhoods: the lanes share the listed entries and lane 0
    walks on from the resume point."""
    w = workloads.sph_lattice_3d(n=3000, seed=21)
    s, cfg = _system(w, f64_mode=1, list_capacity=16)
    s.set_particles_per_warp(8)
    f = w["fields"]
    st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    s.step(1)
    oracle.sph_run(cfg, st, 1)
    assert _rel(s.get("pos"), st.pos) <= F64_TOL
    assert _rel(s.get("rho"), st.rho) <= F64_TOL
    s.close()


def test_particles_per_warp_overlapped_schedule(pg, oracle):
    """1M particles: the overlapped continuity pass and the momentum pass with 16 particles per warp."""
    w = workloads.sph_lattice_3d(n=1000000, seed=13)
    s, cfg = _system(w, f64_mode=1)
    s.set_particles_per_warp(16)
    assert s.info()["overlap_split"] > 0
    f = w["fields"]
    st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    s.step(1)
    oracle.sph_run(cfg, st, 1)
    assert _rel(s.get("pos"), st.pos) <= F64_TOL
    assert _rel(s.get("rho"), st.rho) <= F64_TOL
    s.close()


def test_particles_per_warp_ieee_stays_bit_exact(pg, oracle):
    """The IEEE mode keeps one thread per particle whatever is asked, so it stays bit-exact."""
    w = workloads.sph_lattice_3d(n=4000, seed=33)
    s, cfg = _system(w, f64_mode=0)
    s.set_particles_per_warp(8)
    assert s.info()["particles_per_warp"] == 32
    f = w["fields"]
    st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    s.step(2)
    oracle.sph_run(cfg, st, 2)
    assert np.array_equal(s.get("pos"), st.pos) and np.array_equal(s.get("rho"), st.rho)
    import prestige_gb300._native as nat
    with pytest.raises(nat.PgError):
        s.set_particles_per_warp(4)
    s.close()


def test_batched_particles_per_warp(pg, oracle):
    systems = workloads.batched_dam_breaks(n_systems=5, nmin=400, nmax=1500, seed=8, f64_mode=1)
    cfgs = [w["config"] for w in systems]
    b = ParticleSystem.batch(cfgs, [w["n"] for w in systems])
    for k in ("pos", "vel", "rho", "mass"):
        b.set(k, np.concatenate([w["fields"][k] for w in systems]))
    b.set_particles_per_warp(8)
    b.step(1)
    pos = b.get("pos")
    off = 0
    for w in systems:
        f = w["fields"]
        st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
        oracle.sph_run(w["config"], st, 1)
        assert _rel(pos[off:off + w["n"]], st.pos) <= F64_TOL
        off += w["n"]
    b.close()
