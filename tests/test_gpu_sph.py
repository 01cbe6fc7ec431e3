"""SPH pair pass + integrator on the GPU vs the CPU oracle.

Tolerances
  IEEE modes (f64 native, f32 exact): bit-exact (same operation order, no contraction).
  f64 fast mode (double-word arithmetic on the FP32 pipe): normwise relative error per step
      max_i |a_gpu - a_ref| / max_i |a_ref| <= 1e-10, same for drho; positions after a step
      within 1e-10 of max |x|.
  f32 fast mode (fused multiply-add): normwise 1e-4.
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


def _pair(w, precision=1, f64_mode=0):
    cfg = dict(w["config"])
    cfg["precision"] = precision
    cfg["f64_mode"] = f64_mode
    s = ParticleSystem(make_config(**cfg), w["n"])
    f = w["fields"]
    dt = np.float64 if precision == 1 else np.float32
    for k in ("pos", "vel", "rho", "mass"):
        s.set(k, np.asarray(f[k], dt))
    return s, cfg


def _ostate(oracle, w, f64=True):
    f = w["fields"]
    dt = np.float64 if f64 else np.float32
    return oracle.SphState(np.asarray(f["pos"], dt), np.asarray(f["vel"], dt), np.asarray(f["rho"], dt),
                           np.asarray(f["mass"], dt), f64=f64)


WORK = [
    ("lattice3d", lambda: workloads.sph_lattice_3d(n=4096, seed=2)),
    ("lattice3d_half", lambda: workloads.sph_lattice_3d(n=3000, seed=9, cell_multiplier=0.5)),
    ("dam2d", lambda: workloads.dam_break_2d(dx=0.05)),
]


@pytest.mark.parametrize("name,make", WORK)
def test_rates_f64_native_bit_exact(pg, oracle, name, make):
    w = make()
    s, cfg = _pair(w, 1, 0)
    acc, drho = s.compute_rates()
    oacc, odrho = oracle.sph_rates(cfg, _ostate(oracle, w))
    assert np.array_equal(acc, oacc)
    assert np.array_equal(drho, odrho)


@pytest.mark.parametrize("name,make", WORK)
def test_rates_f32_exact_bit_exact(pg, oracle, name, make):
    w = make()
    s, cfg = _pair(w, 0, 0)
    acc, drho = s.compute_rates()
    oacc, odrho = oracle.sph_rates(cfg, _ostate(oracle, w, f64=False))
    assert np.array_equal(acc, oacc)
    assert np.array_equal(drho, odrho)


@pytest.mark.parametrize("name,make", WORK)
def test_rates_f64_fast_within_tolerance(pg, oracle, name, make):
    w = make()
    s, cfg = _pair(w, 1, 1)
    acc, drho = s.compute_rates()
    oacc, odrho = oracle.sph_rates(cfg, _ostate(oracle, w))
    assert _rel(acc, oacc) <= F64_TOL
    assert _rel(drho, odrho) <= F64_TOL


@pytest.mark.parametrize("name,make", WORK)
def test_rates_f32_fast(pg, oracle, name, make):
    w = make()
    s, cfg = _pair(w, 0, 1)
    acc, drho = s.compute_rates()
    oacc, odrho = oracle.sph_rates(cfg, _ostate(oracle, w, f64=False))
    assert _rel(acc, oacc) <= 1e-4
    assert _rel(drho, odrho) <= 1e-4


@pytest.mark.parametrize("name,make", WORK)
def test_steps_f64_native_bit_exact(pg, oracle, name, make):
    w = make()
    s, cfg = _pair(w, 1, 0)
    st = _ostate(oracle, w)
    for _ in range(3):
        s.step(2)
        oracle.sph_run(cfg, st, 2)
        assert np.array_equal(s.get("pos"), st.pos)
        assert np.array_equal(s.get("vel"), st.vel)
        assert np.array_equal(s.get("rho"), st.rho)


@pytest.mark.parametrize("name,make", WORK)
def test_step_f64_fast_per_step(pg, oracle, name, make):
    """Each step from the same state: positions, velocities, densities within the f64 bound."""
    w = make()
    s, cfg = _pair(w, 1, 1)
    st = _ostate(oracle, w)
    for _ in range(3):
        s.step(1)
        oracle.sph_run(cfg, st, 1)
        assert _rel(s.get("pos"), st.pos) <= F64_TOL
        dv = np.abs(s.get("vel") - st.vel).max()
        assert dv <= F64_TOL * max(np.abs(st.vel).max(), cfg["dt"] * 1e3)
        assert _rel(s.get("rho"), st.rho) <= F64_TOL
        # restart both from the oracle state so the bound is per step
        s.set("pos", st.pos)
        s.set("vel", st.vel)
        s.set("rho", st.rho)


def test_graph_replay_matches_eager(pg):
    w = workloads.sph_lattice_3d(n=5000, seed=4)
    a, _ = _pair(w, 1, 0)
    b, _ = _pair(w, 1, 0)
    b.enable_graph(True)
    a.step(5)
    b.step(5)
    assert np.array_equal(a.get("pos"), b.get("pos"))
    assert np.array_equal(a.get("rho"), b.get("rho"))


def test_dam_break_walls_fixed(pg):
    w = workloads.dam_break_2d(dx=0.05)
    s, cfg = _pair(w, 1, 0)
    p0 = s.get("pos")
    s.step(20)
    p1 = s.get("pos")
    nf = w["n_fluid"]
    assert np.array_equal(p0[nf:], p1[nf:])
    assert not np.array_equal(p0[:nf], p1[:nf])
    assert np.isfinite(p1).all()


def test_errors_are_reported(pg):
    import prestige_gb300._native as nat
    s = ParticleSystem(make_config(dim=3, h=0.01, tait_B=1e4), 10)
    with pytest.raises(nat.PgError) as e:
        s.set("pos", np.zeros(7))
    assert e.value.status == nat.PG_EINVAL
    with pytest.raises(nat.PgError) as e:
        s.get("nope")
    assert e.value.status == nat.PG_ENOTFOUND
    with pytest.raises(nat.PgError):
        ParticleSystem(make_config(dim=4), 10)


@pytest.mark.parametrize("cap", [4, 16, 48])
@pytest.mark.parametrize("precision,mode", [(1, 0), (0, 0), (1, 1)])
def test_list_overflow_continues_the_walk(pg, oracle, cap, precision, mode):
    """Neighbour lists shorter than the neighbour count: the pair passes finish the candidate
    walk from where the list stopped, in the same order, so results are unchanged.  (About 74
    neighbours: with 4 and 16 entries every list stops among the lower slots, with 48 among the
    upper ones, so in the IEEE mode some pairs have their value stored on one side only.)"""
    w = workloads.sph_lattice_3d(n=3000, seed=21)
    cfg = dict(w["config"])
    cfg.update(precision=precision, f64_mode=mode, list_capacity=cap)
    s = ParticleSystem(make_config(**cfg), w["n"])
    f64 = precision == 1
    dt = np.float64 if f64 else np.float32
    for k in ("pos", "vel", "rho", "mass"):
        s.set(k, np.asarray(w["fields"][k], dt))
    acc, drho = s.compute_rates()
    oacc, odrho = oracle.sph_rates(cfg, _ostate(oracle, w, f64=f64))
    st = _ostate(oracle, w, f64=f64)
    s.step(2)
    oracle.sph_run(cfg, st, 2)
    if mode == 0:
        assert np.array_equal(acc, oacc) and np.array_equal(drho, odrho)
        assert np.array_equal(s.get("pos"), st.pos) and np.array_equal(s.get("rho"), st.rho)
    else:
        assert _rel(acc, oacc) <= F64_TOL and _rel(drho, odrho) <= F64_TOL
        assert _rel(s.get("pos"), st.pos) <= F64_TOL


@pytest.mark.parametrize("mult", [0.4, 0.5, 1.0])
def test_steps_bit_exact_across_cell_sizes(pg, oracle, mult):
    """The neighbour lists and pair passes give the oracle's results for cell multipliers with
    reach 1, 2 and 3 (cell sizes 2h, h and 0.8h)."""
    w = workloads.sph_lattice_3d(n=4000, seed=41, cell_multiplier=mult)
    s, cfg = _pair(w, 1, 0)
    st = _ostate(oracle, w)
    s.step(2)
    oracle.sph_run(cfg, st, 2)
    assert np.array_equal(s.get("pos"), st.pos)
    assert np.array_equal(s.get("rho"), st.rho)
    assert s.info()["reach"] == (3 if mult == 0.4 else 2 if mult == 0.5 else 1)


def test_overlapped_continuity_and_lists_match_the_oracle(pg, oracle):
    """From 1M particles a double-word step runs the continuity pass over the first 70 % of the
    slots beside the neighbour lists of the rest (two streams); the step must still match the
    oracle, and replaying it as a CUDA graph must give the same bits."""
    w = workloads.sph_lattice_3d(n=1000000, seed=13)
    s, cfg = _pair(w, 1, 1)
    assert s.info()["overlap_split"] > 0
    st = _ostate(oracle, w)
    s.step(2)
    oracle.sph_run(cfg, st, 2)
    assert _rel(s.get("pos"), st.pos) <= F64_TOL
    assert _rel(s.get("rho"), st.rho) <= F64_TOL
    assert _rel(s.get("vel"), st.vel) <= F64_TOL
    g, _ = _pair(w, 1, 1)
    g.enable_graph(True)
    g.step(2)
    assert np.array_equal(g.get("pos"), s.get("pos")) and np.array_equal(g.get("rho"), s.get("rho"))


def test_overlapped_schedule_with_list_overflow(pg, oracle):
    """The overlapped schedule (1M particles) with lists too short for the neighbourhoods: the
    passes finish every overflowed list by walking on, in both slot ranges."""
    w = workloads.sph_lattice_3d(n=1000000, seed=17)
    cfg = dict(w["config"])
    cfg.update(precision=1, f64_mode=1, list_capacity=24)
    s = ParticleSystem(make_config(**cfg), w["n"])
    for k in ("pos", "vel", "rho", "mass"):
        s.set(k, np.asarray(w["fields"][k], np.float64))
    assert s.info()["overlap_split"] > 0
    st = _ostate(oracle, w)
    s.step(1)
    oracle.sph_run(cfg, st, 1)
    assert _rel(s.get("pos"), st.pos) <= F64_TOL
    assert _rel(s.get("rho"), st.rho) <= F64_TOL


def _df_split(x):
    hi = np.float32(x)
    return hi, np.float32(x - np.float64(hi))


def test_fast_mode_pair_below_double_word_resolution(pg, oracle):
    """Two particles whose f64 positions differ but whose shifted double-word positions
    (x - min + 8 h) are the same: the exact lists keep the pair (f64 r^2 > 0), the double-word
    passes cannot resolve it and skip it, and the continuity pass writes a zero per-entry cache
    entry for it, so the momentum pass adds nothing for it rather than the entry a previous step
    left there.  The step stays within the f64 bound of the oracle, which keeps the pair."""
    w = workloads.sph_lattice_3d(n=4096, seed=2)
    s, cfg = _pair(w, 1, 1)
    s.step(1)  # the per-entry cache now holds this step's entries
    f = w["fields"]
    pos = np.array(f["pos"], np.float64)
    i, j = 100, 101
    pad = 8.0 * cfg["h"]
    moved = None
    for delta in (2e-16, 1e-16, 5e-17, 2e-17, 1e-17):
        b = pos[i].copy()
        b[0] += delta
        if b[0] == pos[i][0]:
            continue
        trial = pos.copy()
        trial[j] = b
        mins = trial.min(axis=0)
        xa, xb = (trial[i] - mins) + pad, (trial[j] - mins) + pad
        if all(_df_split(xa[c]) == _df_split(xb[c]) for c in range(3)):
            moved = trial
            break
    assert moved is not None, "no separation below the double-word resolution found"
    d = moved[i] - moved[j]
    assert 0.0 < float(d @ d) < (2.0 * cfg["h"]) ** 2
    vel = np.asarray(f["vel"], np.float64)
    rho = np.asarray(f["rho"], np.float64)
    s.set("pos", moved)
    s.set("vel", vel)
    s.set("rho", rho)
    st = oracle.SphState(moved, vel, rho, np.asarray(f["mass"], np.float64))
    s.step(1)
    oracle.sph_run(cfg, st, 1)
    assert _rel(s.get("pos"), st.pos) <= F64_TOL
    dv = np.abs(s.get("vel") - st.vel).max()
    assert dv <= F64_TOL * max(np.abs(st.vel).max(), cfg["dt"] * 1e3)
    assert _rel(s.get("rho"), st.rho) <= F64_TOL
    s.close()


@pytest.mark.parametrize("cap", [128, 24])
def test_ieee_overlapped_lists_match_the_oracle_bit_exact(pg, oracle, cap):
    """From 1M particles the IEEE step builds the lists of the last three quarters of the slots
    on a second stream beside the pair values of the first-quarter slots whose partners all lie
    in the first quarter; the rest follow once every list is built.  Bit-exact with the oracle,
    also with lists too short for the neighbourhoods (pairs held by one list only, continued
    walks), and the same bits replayed from a CUDA graph."""
    w = workloads.sph_lattice_3d(n=1000000, seed=19)
    cfg = dict(w["config"])
    cfg.update(precision=1, f64_mode=0, list_capacity=cap)
    s = ParticleSystem(make_config(**cfg), w["n"])
    workloads.load_into(s, w)
    assert s.info()["overlap_split"] > 0
    st = _ostate(oracle, w)
    s.step(1)
    oracle.sph_run(cfg, st, 1)
    assert np.array_equal(s.get("pos"), st.pos) and np.array_equal(s.get("rho"), st.rho)
    assert np.array_equal(s.get("vel"), st.vel)
    g = ParticleSystem(make_config(**cfg), w["n"])
    workloads.load_into(g, w)
    g.enable_graph(True)
    g.step(1)
    assert np.array_equal(g.get("pos"), s.get("pos")) and np.array_equal(g.get("rho"), s.get("rho"))


@pytest.mark.parametrize("cap", [4, 16, 48, 128])
def test_pair_once_ieee_bit_exact(pg, oracle, cap):
    """The IEEE step evaluates each pair once from 16,384 particles (below, the two-sided passes
    run).  3D lattice of 20,000 particles, bit-exact with the oracle over two steps, with lists
    cut at 4, 16 or 48 entries (about 74 neighbours: pairs held by one list only, continued
    walks) and with full lists."""
    w = workloads.sph_lattice_3d(n=20000, seed=23)
    cfg = dict(w["config"])
    cfg.update(precision=1, f64_mode=0, list_capacity=cap)
    s = ParticleSystem(make_config(**cfg), w["n"])
    workloads.load_into(s, w)
    st = _ostate(oracle, w)
    s.step(2)
    oracle.sph_run(cfg, st, 2)
    assert np.array_equal(s.get("pos"), st.pos) and np.array_equal(s.get("rho"), st.rho)
    assert np.array_equal(s.get("vel"), st.vel)


def test_pair_once_ieee_2d_dam_break_bit_exact(pg, oracle):
    """The pair-once IEEE kernels in 2D with walls: the dam break at dx = 0.01 (20,000 fluid
    particles and the wall layers), bit-exact with the oracle over three steps."""
    w = workloads.dam_break_2d(dx=0.01)
    assert w["n"] >= 16384
    s, cfg = _pair(w, 1, 0)
    st = _ostate(oracle, w)
    s.step(3)
    oracle.sph_run(cfg, st, 3)
    assert np.array_equal(s.get("pos"), st.pos) and np.array_equal(s.get("rho"), st.rho)
    assert np.array_equal(s.get("vel"), st.vel)
