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
