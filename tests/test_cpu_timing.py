"""The CPU timing build (oracle/cpu_timing.cpp, the CPU baseline bench.py times) computes the
oracle's step: per step within 1e-10 normwise of the parity build in f64 (it is compiled with
floating-point contraction allowed, so on a host with fused multiply-add the last bits differ),
on 3D lattices with cell multipliers 1 and 1/2 and on the 2D dam break with its fixed walls."""
import numpy as np
import pytest

from prestige_gb300 import workloads

F64_TOL = 1e-10


def _state(oracle, w, f64=True):
    f = w["fields"]
    dt = np.float64 if f64 else np.float32
    return oracle.SphState(np.asarray(f["pos"], dt), np.asarray(f["vel"], dt), np.asarray(f["rho"], dt),
                           np.asarray(f["mass"], dt), f64=f64)


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


CASES = [
    ("lattice", lambda: workloads.sph_lattice_3d(n=6000, seed=2)),
    ("lattice_half_cells", lambda: workloads.sph_lattice_3d(n=6000, seed=3, cell_multiplier=0.5)),
    ("dam_break", lambda: workloads.dam_break_2d(dx=0.05)),
]


@pytest.mark.parametrize("name,make", CASES)
def test_timing_build_matches_the_oracle_per_step(oracle, name, make):
    w = make()
    cfg = w["config"]
    ref = _state(oracle, w)
    fast = _state(oracle, w)
    for _ in range(3):
        oracle.sph_run(cfg, ref, 1)
        oracle.sph_run_timing(cfg, fast, 1)
        assert _rel(fast.pos, ref.pos) <= F64_TOL
        assert np.abs(fast.vel - ref.vel).max() <= F64_TOL * max(np.abs(ref.vel).max(), cfg["dt"] * 1e3)
        assert _rel(fast.rho, ref.rho) <= F64_TOL
        for c in range(len(ref.cols)):  # restart from the parity state: the bound is per step
            fast.cols[c][:] = ref.cols[c]
    if "n_fluid" in w:
        assert np.array_equal(fast.pos[w["n_fluid"]:], w["fields"]["pos"][w["n_fluid"]:])


def test_timing_build_f32(oracle):
    w = workloads.sph_lattice_3d(n=5000, seed=4)
    ref = _state(oracle, w, f64=False)
    fast = _state(oracle, w, f64=False)
    oracle.sph_run(w["config"], ref, 2)
    oracle.sph_run_timing(w["config"], fast, 2)
    assert _rel(fast.pos, ref.pos) <= 1e-5
    assert _rel(fast.rho, ref.rho) <= 1e-5


def test_timing_build_list_capacity_grows(oracle):
    """A neighbourhood denser than the first list capacity (128 in 3D): the lists are rebuilt
    with a larger capacity and the step still matches the oracle."""
    w = workloads.sph_lattice_3d(n=4000, seed=5, dx=0.006)
    w["config"]["h"] = 0.013 * 1.6  # about 800 neighbours per particle, ten times the usual
    w["config"]["dt"] = 0.25 * w["config"]["h"] / w["config"]["c0"]
    ref = _state(oracle, w)
    fast = _state(oracle, w)
    oracle.sph_run(w["config"], ref, 1)
    oracle.sph_run_timing(w["config"], fast, 1)
    assert _rel(fast.pos, ref.pos) <= F64_TOL
    assert _rel(fast.rho, ref.rho) <= F64_TOL
