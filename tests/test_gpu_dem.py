"""DEM contact pass + integrator on the GPU vs the CPU oracle (bit-exact, IEEE double).

Cases: a compressed lattice where every sphere touches its neighbours and the walls (normal,
tangential history, Coulomb slip and torques all active), the RSA settling workload at small
size, and the contact-slot overflow, which must be reported as PG_EOVERFLOW while the physics
stays identical to the oracle's (both drop the extra history entries).
"""
import numpy as np
import pytest

import prestige_gb300._native as nat
from prestige_gb300 import ParticleSystem, make_config, workloads

pytestmark = pytest.mark.gpu


def compressed_lattice(nside=(8, 8, 8), r=0.5e-3, overlap=0.02, seed=0, capacity=16):
    return workloads.dem_compressed_lattice(nside=nside, r=r, overlap=overlap, seed=seed, capacity=capacity)


def _run_pair(w, steps, chunk):
    cfg = w["config"]
    s = ParticleSystem(make_config(**cfg), w["n"])
    workloads.load_into(s, w)
    return s


def _ostate(oracle, w):
    f = w["fields"]
    return oracle.DemState(f["pos"], f["vel"], f["omega"], f["radius"], f["mass"], w["config"]["contact_capacity"])


@pytest.mark.parametrize("graph", [False, True])
def test_dem_compressed_lattice_bit_exact(pg, oracle, graph):
    w = compressed_lattice()
    s = _run_pair(w, 0, 0)
    if graph:
        s.enable_graph(True)
    st = _ostate(oracle, w)
    for _ in range(4):
        s.step(5)
        c, _ = oracle.dem_run(w["config"], st, 5)
        assert c > 0
        assert s.dem_contacts() == c
        assert np.array_equal(s.get("pos"), st.pos)
        assert np.array_equal(s.get("vel"), st.vel)
        assert np.array_equal(s.get("omega"), st.omega)
        pid, xi = s.dem_history()
        assert np.array_equal(pid.reshape(-1), st.hpid)
        assert np.array_equal(xi.reshape(-1), st.hxi)


def test_dem_rsa_settling_small(pg, oracle):
    """Free spheres (the contact-free shortcuts of the integrator), some spinning, some with a
    signed-zero spin component, a few touching the floor."""
    w = workloads.dem_settling(n=3000, box=(0.02, 0.02, 0.06), seed=1)
    rng = np.random.default_rng(4)
    om = rng.normal(0.0, 20.0, size=(w["n"], 3))
    om[::7] = 0.0
    om[1::7, 0] = -0.0
    w["fields"]["omega"] = om
    pos = np.array(w["fields"]["pos"], copy=True)
    low = np.argsort(pos[:, 2])[:20]
    pos[low, 2] = w["fields"]["radius"][low] * (1.0 - 1e-3)  # slightly into the floor
    w["fields"]["pos"] = pos
    s = _run_pair(w, 0, 0)
    st = _ostate(oracle, w)
    s.step(10)
    oracle.dem_run(w["config"], st, 10)
    assert np.array_equal(s.get("pos"), st.pos)
    assert np.array_equal(s.get("vel"), st.vel)
    got = np.ascontiguousarray(s.get("omega"), np.float64).reshape(-1).view(np.uint64)
    ref = np.ascontiguousarray(st.omega, np.float64).reshape(-1).view(np.uint64)
    assert np.array_equal(got, ref)  # signs of zeros too
    pid, xi = s.dem_history()
    assert np.array_equal(pid.reshape(-1), st.hpid)
    assert np.array_equal(xi.reshape(-1), st.hxi)


def test_dem_contact_overflow_reported(pg, oracle):
    w = compressed_lattice(nside=(5, 5, 5), capacity=2)
    s = _run_pair(w, 0, 0)
    st = _ostate(oracle, w)
    with pytest.raises(nat.PgError) as e:
        s.step(1)
    assert e.value.status == nat.PG_EOVERFLOW
    c, _ = oracle.dem_run(w["config"], st, 1)
    assert c == -1
    assert np.array_equal(s.get("pos"), st.pos)
    assert np.array_equal(s.get("vel"), st.vel)


@pytest.mark.parametrize("overlap", [0.4, 0.5])
def test_dem_more_contacts_than_the_walk_buffer(pg, oracle, overlap):
    """Lattices so compressed that many spheres have 17 to 29 contacts (walls included): the
    walk's per-thread contact buffer (16 entries) fills, the lane evaluates the first contacts
    itself before walking on, and the warp evaluates the rest; bit-exact with the oracle."""
    w = compressed_lattice(nside=(6, 6, 6), overlap=overlap, capacity=32)
    s = _run_pair(w, 0, 0)
    st = _ostate(oracle, w)
    for _ in range(2):
        s.step(1)
        c, _ = oracle.dem_run(w["config"], st, 1)
        assert s.dem_contacts() == c
        assert np.array_equal(s.get("pos"), st.pos)
        assert np.array_equal(s.get("vel"), st.vel)
        assert np.array_equal(s.get("omega"), st.omega)
        pid, xi = s.dem_history()
        assert np.array_equal(pid.reshape(-1), st.hpid)
        assert np.array_equal(xi.reshape(-1), st.hxi)
    assert ((pid != 0xFFFFFFFF).sum(axis=1) > 16).any()
