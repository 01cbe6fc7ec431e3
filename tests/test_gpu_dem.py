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
    rng = np.random.default_rng(seed)
    sp = 2 * r * (1 - overlap)
    idx = np.stack(np.meshgrid(*[np.arange(k) for k in nside], indexing="ij"), -1).reshape(-1, 3)
    pos = (idx + 0.5) * sp + rng.uniform(-0.05, 0.05, size=idx.shape) * r
    n = pos.shape[0]
    radius = r * (1 + rng.uniform(-0.05, 0.0, size=n))
    mass = 2600 * 4 / 3 * np.pi * radius ** 3
    vel = rng.normal(0, 0.05, size=(n, 3))
    omega = rng.normal(0, 50.0, size=(n, 3))
    box = np.array(nside) * sp
    cfg = dict(model=1, dim=3, precision=1, domain_lo=[-2e-3] * 3, domain_hi=list(box + 2e-3), cell_multiplier=1.0,
               gravity=[0, 0, -9.81], dt=1e-6, kn=1e5, restitution=0.9, mu=0.3, kt=1e5 * 2 / 7, r_max=r,
               wall_lo=[0, 0, 0], wall_hi=list(box - 0.01 * r), contact_capacity=capacity)
    fields = {"pos": pos, "vel": vel, "omega": omega, "radius": radius, "mass": mass}
    return {"config": cfg, "n": n, "fields": fields}


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
    w = workloads.dem_settling(n=3000, box=(0.02, 0.02, 0.06), seed=1)
    s = _run_pair(w, 0, 0)
    st = _ostate(oracle, w)
    s.step(10)
    oracle.dem_run(w["config"], st, 10)
    assert np.array_equal(s.get("pos"), st.pos)
    assert np.array_equal(s.get("vel"), st.vel)


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
