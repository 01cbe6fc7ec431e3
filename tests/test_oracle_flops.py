"""Flop census of the oracle's SPH step (each +, -, *, / and sqrt one flop).

bench.py reports flops per particle-step as (neighbour pairs per particle) x (flops per
continuity pair + flops per momentum pair) + flops per particle, with the per-pair and
per-particle figures fixed as constants.  This recomputes them from the oracle on the sample
the constants name and checks the census's own bookkeeping: a step's flops are its two pair
loops plus the per-particle terms, and the loops split exactly into candidate tests and pair
terms.
"""
import importlib.util
import os

import numpy as np
import pytest

from oracle import py_oracle as po
from prestige_gb300 import workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_consts", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _census(n, seed=2):
    w = workloads.sph_lattice_3d(n=n, seed=seed)
    f = w["fields"]
    st = po.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    before = [c.copy() for c in st.cols]
    c = po.sph_flop_census(w["config"], st)
    assert all(np.array_equal(a, b) for a, b in zip(before, st.cols))  # the census leaves the state alone
    return w, c


def _per_pair(c):
    rejected = c["candidates"] - c["pairs"]
    cont = (c["cont_loops"] - c["test_flops"] * rejected) / c["pairs"]
    mom = (c["mom_loops"] - c["test_flops"] * rejected) / c["pairs"]
    per_particle = (c["step"] - c["cont_loops"] - c["mom_loops"]) / c["particles"]
    return cont, mom, per_particle


def test_bench_flop_constants_match_the_oracle_census():
    b = _bench()
    w, c = _census(b.FLOPS_SAMPLE_PARTICLES)
    cont, mom, per_particle = _per_pair(c)
    assert cont == pytest.approx(b.FLOPS_PER_PAIR["continuity"], rel=2e-5)
    assert mom == pytest.approx(b.FLOPS_PER_PAIR["momentum"], rel=2e-5)
    assert per_particle == b.FLOPS_PER_PARTICLE


def test_census_bookkeeping_and_branch_bounds():
    w, c = _census(4096, seed=3)
    n = w["n"]
    assert c["particles"] == n and c["test_flops"] == 8
    # every particle is its own candidate and is never its own pair
    assert c["candidates"] >= c["pairs"] + n
    cont, mom, per_particle = _per_pair(c)
    # continuity pair: d 3, r^2 5, r 1, q 1, F 3 (q < 1) or 4, v_ij 3, w 5, m_j (w F) 2, sum 1
    assert 24.0 <= cont <= 25.0
    # momentum pair: d, r^2, r, q, F as above (13 or 14), v_ij and w 8, viscosity 5 when w < 0,
    # (P_i + P_j) + Pi_ij 2, times F and m_j 2, three (mul, sub) 6
    assert 31.0 <= mom <= 37.0
    # Tait (gamma = 7: 6 powers, rho/rho0, -1, *B, rho^2, /) 11, rho update 2, v and x 5 per axis
    assert per_particle == 11 + 2 + 15
    # integer counts: the flops are whole numbers
    for k in ("cont_loops", "mom_loops", "step"):
        assert c[k] == int(c[k])


def test_census_scales_with_pairs():
    """Per-pair flops depend only on the branch mix, not on the sample size."""
    _, a = _census(4096, seed=2)
    _, b = _census(32768, seed=2)
    ca, ma, _ = _per_pair(a)
    cb, mb, _ = _per_pair(b)
    assert ca == pytest.approx(cb, rel=2e-3) and ma == pytest.approx(mb, rel=2e-3)
