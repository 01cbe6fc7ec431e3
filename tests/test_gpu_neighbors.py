"""Neighbour search on the GPU vs the CPU oracle: bit-exact integer results.

Covers the cell hash, the stable (cell, id) ordering, the cell-start table, neighbour counts
and CSR lists, and the reference's eq1 gather `force[i] += mass[j]` (prestige/src/lib.rs:7-12)
over the neighbour set.  Edge cases: one particle, particles outside the grid box (clamped),
coincident particles, 2D and 3D, f32 and f64, cell multipliers 1 and 0.5.
"""
import numpy as np
import pytest

from prestige_gb300 import ParticleSystem, make_config, workloads

pytestmark = pytest.mark.gpu


def _system(w, f64=True):
    cfg = dict(w["config"])
    cfg["precision"] = 1 if f64 else 0
    s = ParticleSystem(make_config(**cfg), w["n"])
    workloads.load_into(s, w)
    return s, cfg


CASES = [
    ("lattice3d", lambda: workloads.sph_lattice_3d(n=3000, seed=7)),
    ("lattice3d_half", lambda: workloads.sph_lattice_3d(n=2500, seed=8, cell_multiplier=0.5)),
    ("dam2d", lambda: workloads.dam_break_2d(dx=0.1)),
]


@pytest.mark.parametrize("f64", [True, False])
@pytest.mark.parametrize("name,make", CASES)
def test_cell_list_bit_exact(pg, oracle, name, make, f64):
    w = make()
    s, cfg = _system(w, f64)
    cell, ids, start = s.neighbors()
    support = 2.0 * cfg["h"]
    ocell, oid, ostart = oracle.cell_list(w["fields"]["pos"], cfg["domain_lo"], cfg["domain_hi"], support,
                                          cfg["cell_multiplier"], f64)
    assert np.array_equal(ids, oid)
    assert np.array_equal(cell, ocell[oid])
    assert np.array_equal(start, ostart)
    # stable order: (cell, id) lexicographic
    order = np.lexsort((np.arange(w["n"]), ocell))
    assert np.array_equal(ids, order)


@pytest.mark.parametrize("f64", [True, False])
@pytest.mark.parametrize("name,make", CASES)
def test_neighbor_counts_and_lists(pg, oracle, name, make, f64):
    w = make()
    s, cfg = _system(w, f64)
    support = 2.0 * cfg["h"]
    args = (w["fields"]["pos"], cfg["domain_lo"], cfg["domain_hi"], support, cfg["cell_multiplier"], f64)
    assert np.array_equal(s.count_neighbors(), oracle.neighbor_counts(*args))
    offs, nbr = s.neighbor_list()
    ooffs, onbr = oracle.neighbor_list(*args)
    assert np.array_equal(offs, ooffs)
    assert np.array_equal(nbr, onbr)


def test_neighbors_brute_force(pg):
    """Neighbour sets equal an all-pairs search (the reference's j loop, simple_cpu.rs:8)."""
    w = workloads.sph_lattice_3d(n=800, seed=3)
    s, cfg = _system(w)
    pos = w["fields"]["pos"]
    offs, nbr = s.neighbor_list()
    d = pos[:, None, :] - pos[None, :, :]
    r2 = (d ** 2).sum(-1)
    near = r2 < (2 * cfg["h"]) ** 2
    for i in range(w["n"]):
        got = set(nbr[offs[i]:offs[i + 1]].tolist())
        assert got == set(np.nonzero(near[i])[0].tolist())


def test_outside_box_and_coincident(pg, oracle):
    rng = np.random.default_rng(11)
    n = 600
    pos = rng.uniform(-0.3, 1.3, size=(n, 3))   # many outside the [0,1]^3 grid box
    pos[10] = pos[11]                           # coincident pair
    pos[20] = [1e3, -1e3, 5.0]                  # far outside
    cfg = dict(model=0, dim=3, precision=1, h=0.06, domain_lo=[0, 0, 0], domain_hi=[1, 1, 1], tait_B=1e4)
    s = ParticleSystem(make_config(**cfg), n)
    s.set("pos", pos)
    cell, ids, start = s.neighbors()
    ocell, oid, ostart = oracle.cell_list(pos, [0, 0, 0], [1, 1, 1], 0.12, 1.0, True)
    assert np.array_equal(ids, oid) and np.array_equal(start, ostart)
    assert np.array_equal(s.count_neighbors(), oracle.neighbor_counts(pos, [0, 0, 0], [1, 1, 1], 0.12, 1.0, True))


def test_single_particle(pg):
    s = ParticleSystem(make_config(dim=3, h=0.1, tait_B=1e4), 1)
    s.set("pos", np.array([[0.5, 0.5, 0.5]]))
    cell, ids, start = s.neighbors()
    assert ids.tolist() == [0]
    assert s.count_neighbors().tolist() == [1]


@pytest.mark.parametrize("name,make", CASES)
def test_eq1_gather_sum(pg, oracle, name, make):
    """force[i] += mass[j] over neighbours, integer masses -> exact; any masses -> bit-exact."""
    w = make()
    s, cfg = _system(w, True)
    n = w["n"]
    rng = np.random.default_rng(5)
    mass_int = rng.integers(1, 9, size=n).astype(np.float64)
    s.set("m_int", mass_int)
    s.set("force", np.zeros(n))
    s.gather_sum("force", "m_int")
    got = s.get("force")
    counts = s.count_neighbors()
    offs, nbr = s.neighbor_list()
    expect = np.array([mass_int[nbr[offs[i]:offs[i + 1]]].sum() for i in range(n)])
    assert np.array_equal(got, expect)
    # random real-valued masses: bit-exact against the oracle's sequential sum
    m = rng.uniform(0.1, 2.0, size=n)
    f0 = rng.normal(size=n)
    s.set("mr", m)
    s.set("fr", f0)
    s.gather_sum("fr", "mr")
    ref = oracle.gather_sum(w["fields"]["pos"], cfg["domain_lo"], cfg["domain_hi"], 2 * cfg["h"], m, f0,
                            cfg["cell_multiplier"], True)
    assert np.array_equal(s.get("fr"), ref)
    assert counts.min() >= 1


def test_cells_at_cell_boundaries(pg, oracle):
    """Coordinates on and within a few ulps of cell boundaries, where the hash's FP32 shortcut
    cannot decide the cell and the f64 formula runs: cells and order stay the oracle's."""
    rng = np.random.default_rng(12)
    lo, hi, h = [-0.3, 0.1, 0.0], [1.7, 2.1, 2.0], 0.05
    cell = 2 * h
    n = 4000
    k = rng.integers(0, 20, size=(n, 3)).astype(np.float64)
    pos = np.array(lo) + k * cell
    ulps = rng.integers(-4, 5, size=(n, 3))
    pos = pos + ulps * np.spacing(np.abs(pos) + 1e-300)
    pos[: n // 4] += rng.uniform(0.0, cell, size=(n // 4, 3))  # a quarter away from boundaries
    cfg = dict(model=0, dim=3, precision=1, h=h, domain_lo=lo, domain_hi=hi, tait_B=1e4)
    s = ParticleSystem(make_config(**cfg), n)
    s.set("pos", pos)
    cells, ids, start = s.neighbors()
    ocell, oid, ostart = oracle.cell_list(pos, lo, hi, 2 * h, 1.0, True)
    assert np.array_equal(ids, oid) and np.array_equal(start, ostart)
    assert np.array_equal(cells, ocell[oid])
