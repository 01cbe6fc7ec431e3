"""The neighbour lists the SPH pair passes read (pg_get_pair_lists) vs the oracle's neighbour lists.

In both f64 modes (IEEE and double-word) the list kernel classifies every candidate exactly: an
FP32 test away from the support radius, the oracle's f64 test in a narrow band around it, so the
pair passes need no neighbour test of their own.  Their lists must equal the oracle's f64
neighbour lists (traversal order, i itself and coincident particles left out), entry for entry.
The cubic spline's gradient vanishes at r = 2h, so a pair misplaced at the boundary would not
show in the rates: these tests compare the lists themselves, on lattices built so that many
pairs sit at r = 2h to the last bit.
"""
import numpy as np
import pytest

from prestige_gb300 import ParticleSystem, make_config, workloads

pytestmark = pytest.mark.gpu


def _boundary_lattice(side, h_over_dx, jitter=0.0, seed=0, cell_multiplier=1.0):
    """Cubic lattice (dx = 0.01) whose support 2h equals a lattice distance: the f64 rounding of
    x_i - x_j decides whether those pairs are neighbours."""
    w = workloads.sph_lattice_3d(n=side ** 3, seed=seed)
    dx = 0.01
    i = np.arange(side ** 3)
    pos = np.stack([i % side, (i // side) % side, i // (side * side)], axis=1).astype(np.float64) * dx + 0.5 * dx
    if jitter:
        pos += np.random.default_rng(seed).uniform(-jitter * dx, jitter * dx, size=pos.shape)
    w["fields"]["pos"] = pos
    w["config"]["h"] = h_over_dx * dx
    w["config"]["dt"] = 0.25 * w["config"]["h"] / w["config"]["c0"]
    w["config"]["cell_multiplier"] = cell_multiplier
    return w


def _outside_box(n=3000, seed=7):
    """A random cloud, many particles outside the [0, 1]^3 grid box (clamped into edge cells),
    one far outside, and coincident pairs."""
    w = workloads.sph_lattice_3d(n=n, seed=seed)
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-0.3, 1.3, size=(n, 3))
    pos[10] = pos[11]
    pos[20] = [1e3, -1e3, 5.0]
    pos[21] = [1e3, -1e3, 5.0 + 0.01]
    w["fields"]["pos"] = pos
    h = 0.06
    w["config"].update(h=h, domain_lo=[0.0] * 3, domain_hi=[1.0] * 3, dt=0.25 * h / w["config"]["c0"])
    return w


CASES = [
    ("two_dx", lambda: _boundary_lattice(14, 1.0)),
    ("two_sqrt2_dx", lambda: _boundary_lattice(12, np.sqrt(2.0))),
    ("sqrt5_dx_half_cells", lambda: _boundary_lattice(12, np.sqrt(5.0) / 2.0, cell_multiplier=0.5)),
    ("two_dx_jitter_1e-12", lambda: _boundary_lattice(12, 1.0, jitter=1e-12, seed=3)),
    ("jittered", lambda: workloads.sph_lattice_3d(n=4096, seed=2)),
    ("dam2d", lambda: workloads.dam_break_2d(dx=0.05)),
    ("outside_box", _outside_box),
    ("outside_box_half_cells", lambda: dict(_outside_box(), config=dict(_outside_box()["config"], cell_multiplier=0.5))),
]


def _system(w, f64_mode):
    cfg = dict(w["config"])
    cfg.update(precision=1, f64_mode=f64_mode)
    s = ParticleSystem(make_config(**cfg), w["n"])
    for k in ("pos", "vel", "rho", "mass"):
        s.set(k, np.asarray(w["fields"][k], np.float64))
    return s, cfg


def _oracle_lists(oracle, w, cfg):
    pos = np.asarray(w["fields"]["pos"], np.float64)
    offs, nbr = oracle.neighbor_list(pos, cfg["domain_lo"], cfg["domain_hi"], 2.0 * cfg["h"],
                                     cfg.get("cell_multiplier", 1.0))
    owner = np.repeat(np.arange(len(offs) - 1), np.diff(offs.astype(np.int64)))
    d = pos[owner] - pos[nbr]
    r2 = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]
    if pos.shape[1] == 3:
        r2 = r2 + d[:, 2] * d[:, 2]
    keep = r2 > 0.0
    return [nbr[offs[i]:offs[i + 1]][keep[offs[i]:offs[i + 1]]] for i in range(len(offs) - 1)]


def _pass_lists(s):
    s.compute_rates()
    lengths, entries = s.pair_lists()
    _, ids, _ = s.neighbors()  # same positions, so the same sorted order as the lists
    cap = entries.shape[1]
    assert lengths.max() <= cap, "test case overflows the list capacity"
    out = [None] * s.n
    for k in range(s.n):
        out[ids[k]] = ids[entries[k, :lengths[k]]]
    return out


@pytest.mark.parametrize("mode", [1, 0])
@pytest.mark.parametrize("name,make", CASES)
def test_f64_lists_are_the_exact_neighbours(pg, oracle, name, make, mode):
    w = make()
    s, cfg = _system(w, mode)
    got = _pass_lists(s)
    ref = _oracle_lists(oracle, w, cfg)
    bad = [i for i in range(w["n"]) if not np.array_equal(got[i], ref[i])]
    assert not bad, "particle %d: %s vs %s" % (bad[0], got[bad[0]], ref[bad[0]])


def test_boundary_cases_exercise_the_band(pg, oracle):
    """The two_dx lattice has pairs on both sides of r = 2h after f64 rounding: some axis pairs at
    2 dx are neighbours and some are not."""
    w = _boundary_lattice(14, 1.0)
    pos = w["fields"]["pos"]
    d = pos[:-2] - pos[2:]  # x-neighbours two apart (same row except at row ends)
    r2 = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]
    four_h2 = (2.0 * w["config"]["h"]) * (2.0 * w["config"]["h"])
    row = np.abs(d[:, 1]) + np.abs(d[:, 2]) == 0
    assert (r2[row] < four_h2).any() and (r2[row] >= four_h2).any()


def test_pair_lists_errors(pg):
    from prestige_gb300 import _native as nat
    w = workloads.sph_lattice_3d(n=512, seed=1)
    s, _ = _system(w, 1)
    with pytest.raises(nat.PgError):
        s.pair_lists()  # nothing built yet


def test_overflowed_lists_report_full_lengths(pg, oracle):
    """With a list capacity below the neighbour count the lengths still count every neighbour
    and the stored entries are the first `capacity` of the exact list."""
    w = workloads.sph_lattice_3d(n=4096, seed=2)
    cfg = dict(w["config"])
    cfg.update(precision=1, f64_mode=1, list_capacity=20)
    s = ParticleSystem(make_config(**cfg), w["n"])
    for k in ("pos", "vel", "rho", "mass"):
        s.set(k, np.asarray(w["fields"][k], np.float64))
    s.compute_rates()
    lengths, entries = s.pair_lists()
    _, ids, _ = s.neighbors()
    ref = _oracle_lists(oracle, w, cfg)
    assert lengths.max() > 20
    for k in range(w["n"]):
        r = ref[ids[k]]
        assert lengths[k] == len(r)
        m = min(len(r), 20)
        assert np.array_equal(ids[entries[k, :m]], r[:m])


def test_pair_counts_are_the_oracle_pair_count(pg, oracle):
    """The list lengths of the double-word mode sum to the oracle's neighbour-pair count (j != i
    within 2h), the figure bench.py multiplies by the per-pair flops."""
    from oracle import py_oracle as po
    w = workloads.sph_lattice_3d(n=4096, seed=2)
    s, cfg = _system(w, 1)
    s.compute_rates()
    counts = s.pair_counts()
    lengths, _ = s.pair_lists()
    assert np.array_equal(counts, lengths)
    f = w["fields"]
    census = po.sph_flop_census(cfg, po.SphState(f["pos"], f["vel"], f["rho"], f["mass"]))
    assert int(counts.sum()) == int(census["pairs"])


def test_measure_fma_peaks(pg):
    from prestige_gb300._native import measure_fma_peaks
    fp64, fp32 = measure_fma_peaks()
    assert np.isfinite(fp64) and np.isfinite(fp32)
    assert 0.0 < fp64 < fp32
