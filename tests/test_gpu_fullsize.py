"""Parity at the full sizes of the benchmark workloads.

  * The 4,096,000-particle jittered lattice that bench.py times (160^3, seed 2):
      IEEE f64: three steps bit-exact against the oracle (checked after the first and third);
      double-word f64: two steps, each from the oracle's state, within 1e-10 normwise per step.
  * The 2D dam break at dx = 0.02 (5,000 fluid + 1,518 wall particles) for its 2,000 steps:
      IEEE f64 bit-exact against the oracle, compared every 200 steps so a failure names the
      step window.
  * DEM at 200,000 spheres, bit-exact: the settling workload (graph-replayed) and the
      contact-dense compressed lattice of the DEM bench.
  * The 512 uneven dam breaks of the batched bench (6.1 M particles) in one handle, IEEE f64.

The oracle runs these on all host threads (about 1 s per 4M-particle step on 16 cores).
"""
import numpy as np
import pytest

from prestige_gb300 import ParticleSystem, make_config, workloads

pytestmark = pytest.mark.gpu

F64_TOL = 1e-10


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _handle(w, f64_mode):
    cfg = dict(w["config"], precision=1, f64_mode=f64_mode)
    s = ParticleSystem(make_config(**cfg), w["n"])
    workloads.load_into(s, w)
    return s, cfg


def _ostate(oracle, w):
    f = w["fields"]
    return oracle.SphState(np.asarray(f["pos"], np.float64), np.asarray(f["vel"], np.float64),
                           np.asarray(f["rho"], np.float64), np.asarray(f["mass"], np.float64))


@pytest.fixture(scope="module")
def lattice_4m():
    return workloads.sph_lattice_3d(n=4096000, seed=2)


def test_lattice_4m_ieee_bit_exact(pg, oracle, lattice_4m):
    w = lattice_4m
    s, cfg = _handle(w, 0)
    assert s.info()["overlap_split"] > 0  # the lists of three quarters beside the first pair values
    st = _ostate(oracle, w)
    for k in (1, 2):
        s.step(k)
        oracle.sph_run(cfg, st, k)
        assert np.array_equal(s.get("pos"), st.pos)
        assert np.array_equal(s.get("vel"), st.vel)
        assert np.array_equal(s.get("rho"), st.rho)
    s.close()


def test_lattice_4m_double_word_per_step(pg, oracle, lattice_4m):
    """The bench's mode and schedule (overlapped lists and continuity pass, per-entry cache),
    eager and replayed as a CUDA graph."""
    w = lattice_4m
    s, cfg = _handle(w, 1)
    assert s.info()["overlap_split"] > 0
    g, _ = _handle(w, 1)
    g.enable_graph(True)
    st = _ostate(oracle, w)
    for _ in range(2):
        s.step(1)
        g.step(1)
        oracle.sph_run(cfg, st, 1)
        assert _rel(s.get("pos"), st.pos) <= F64_TOL
        dv = np.abs(s.get("vel") - st.vel).max()
        assert dv <= F64_TOL * np.abs(st.vel).max()
        assert _rel(s.get("rho"), st.rho) <= F64_TOL
        assert np.array_equal(g.get("pos"), s.get("pos")) and np.array_equal(g.get("rho"), s.get("rho"))
        for k in ("pos", "vel", "rho"):  # both restart from the oracle's state: the bound is per step
            s.set(k, getattr(st, k))
            g.set(k, getattr(st, k))
    s.close()
    g.close()


def test_dam_break_full_size_2000_steps_ieee_bit_exact(pg, oracle):
    w = workloads.dam_break_2d(dx=0.02)
    assert w["n_fluid"] == 5000
    s, cfg = _handle(w, 0)
    st = _ostate(oracle, w)
    p0 = s.get("pos")
    for window in range(10):
        s.step(200)
        oracle.sph_run(cfg, st, 200)
        end = 200 * (window + 1)
        assert np.array_equal(s.get("pos"), st.pos), "positions differ by step %d" % end
        assert np.array_equal(s.get("vel"), st.vel), "velocities differ by step %d" % end
        assert np.array_equal(s.get("rho"), st.rho), "densities differ by step %d" % end
    p1 = s.get("pos")
    nf = w["n_fluid"]
    assert np.array_equal(p0[nf:], p1[nf:])  # walls fixed
    assert p1[:nf, 0].max() > 1.2  # the front has advanced from x = 0.99 m
    s.close()


def _dem_pair(oracle, w):
    s = ParticleSystem(make_config(**w["config"]), w["n"])
    workloads.load_into(s, w)
    f = w["fields"]
    st = oracle.DemState(f["pos"], f["vel"], f["omega"], f["radius"], f["mass"], w["config"]["contact_capacity"])
    return s, st


def _dem_equal(s, st):
    assert np.array_equal(s.get("pos"), st.pos)
    assert np.array_equal(s.get("vel"), st.vel)
    assert np.array_equal(s.get("omega"), st.omega)
    pid, xi = s.dem_history()
    assert np.array_equal(pid.reshape(-1), st.hpid)
    assert np.array_equal(xi.reshape(-1), st.hxi)


def test_dem_settling_200k_bit_exact(pg, oracle):
    """The 200,000-sphere settling workload (random sequential insertion), 20 steps, graph-replayed."""
    w = workloads.dem_settling(200000)
    s, st = _dem_pair(oracle, w)
    s.enable_graph(True)
    s.step(20)
    oracle.dem_run(w["config"], st, 20)
    _dem_equal(s, st)
    s.close()


def test_dem_dense_200k_bit_exact(pg, oracle):
    """200,000 spheres on the compressed lattice of the DEM bench: about 500,000 contacts per step,
    tangential history, Coulomb slip and walls, 6 steps."""
    w = workloads.dem_compressed_lattice(nside=(50, 50, 80))
    s, st = _dem_pair(oracle, w)
    for _ in range(3):
        s.step(2)
        c, _ = oracle.dem_run(w["config"], st, 2)
        assert c > 400000 and s.dem_contacts() == c
        _dem_equal(s, st)
    s.close()


def test_batched_512_dam_breaks_bit_exact(pg, oracle):
    """The 512 uneven dam breaks of the batched bench (6.1 M particles) in one handle, IEEE f64,
    graph-replayed: every system equals the oracle run of that system alone after 2 steps."""
    systems = workloads.batched_dam_breaks()
    assert len(systems) == 512
    cfgs = [dict(w["config"], f64_mode=0) for w in systems]
    b = ParticleSystem.batch(cfgs, [w["n"] for w in systems])
    for k in ("pos", "vel", "rho", "mass"):
        b.set(k, np.concatenate([w["fields"][k] for w in systems]))
    b.enable_graph(True)
    b.step(2)
    pos, vel, rho = b.get("pos"), b.get("vel"), b.get("rho")
    o = 0
    for w in systems:
        f = w["fields"]
        st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
        oracle.sph_run(w["config"], st, 2)
        n = w["n"]
        assert np.array_equal(pos[o:o + n], st.pos) and np.array_equal(vel[o:o + n], st.vel)
        assert np.array_equal(rho[o:o + n], st.rho)
        o += n
    b.close()


@pytest.mark.parametrize("mode,tol", [(0, 0.0), (1, 1e-4)])
def test_lattice_4m_f32(pg, oracle, mode, tol):
    """The 4M lattice in single precision: IEEE f32 bit-exact, contracted f32 within 1e-4, one step."""
    w = workloads.sph_lattice_3d(n=4096000, seed=2, precision=0)
    cfg = dict(w["config"], precision=0, f64_mode=mode)
    s = ParticleSystem(make_config(**cfg), w["n"])
    f = w["fields"]
    for k in ("pos", "vel", "rho", "mass"):
        s.set(k, np.asarray(f[k], np.float32))
    st = oracle.SphState(np.asarray(f["pos"], np.float32), np.asarray(f["vel"], np.float32),
                         np.asarray(f["rho"], np.float32), np.asarray(f["mass"], np.float32), f64=False)
    s.step(1)
    oracle.sph_run(cfg, st, 1)
    if mode == 0:
        assert np.array_equal(s.get("pos"), st.pos) and np.array_equal(s.get("rho"), st.rho)
        assert np.array_equal(s.get("vel"), st.vel)
    else:
        assert _rel(s.get("pos"), st.pos) <= tol and _rel(s.get("rho"), st.rho) <= tol
    s.close()
