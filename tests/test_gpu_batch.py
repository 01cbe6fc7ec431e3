"""Batched SPH: many independent dam breaks of uneven sizes in one handle (pg_batch_create).

Each system keeps its own grid, time step and parameters; the concatenated SoA is stepped by
one set of launches per step.  In the IEEE f64 mode every system must match the oracle run of
that system alone, bit for bit, eager and replayed from a CUDA graph; the double-word mode
within the f64 tolerance.
"""
import numpy as np
import pytest

from prestige_gb300 import ParticleSystem, workloads

pytestmark = pytest.mark.gpu

F64_TOL = 1e-10


def _batch(systems, mode):
    cfgs = []
    for w in systems:
        c = dict(w["config"])
        c["f64_mode"] = mode
        cfgs.append(c)
    b = ParticleSystem.batch(cfgs, [w["n"] for w in systems])
    for k in ("pos", "vel", "rho", "mass"):
        b.set(k, np.concatenate([w["fields"][k] for w in systems]))
    return b


def _oracle_runs(oracle, systems, nsteps):
    out = []
    for w in systems:
        f = w["fields"]
        st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
        oracle.sph_run(w["config"], st, nsteps)
        out.append(st)
    return out


def _small_systems(count=7, seed=5):
    return workloads.batched_dam_breaks(n_systems=count, nmin=150, nmax=1500, seed=seed)


@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_per_system_oracle_bit_exact(pg, oracle, graph):
    systems = _small_systems()
    b = _batch(systems, 0)
    if graph:
        b.enable_graph(True)
    nsteps = 6
    b.step(nsteps)
    ref = _oracle_runs(oracle, systems, nsteps)
    pos, vel, rho = b.get("pos"), b.get("vel"), b.get("rho")
    o = 0
    for w, st in zip(systems, ref):
        n = w["n"]
        assert np.array_equal(pos[o:o + n], st.pos)
        assert np.array_equal(vel[o:o + n], st.vel)
        assert np.array_equal(rho[o:o + n], st.rho)
        o += n
    b.close()


def test_batch_fast_mode_within_tolerance(pg, oracle):
    systems = _small_systems(count=5, seed=8)
    b = _batch(systems, 1)
    b.step(1)
    ref = _oracle_runs(oracle, systems, 1)
    pos, rho = b.get("pos"), b.get("rho")
    o = 0
    for w, st in zip(systems, ref):
        n = w["n"]
        p = pos[o:o + n]
        assert np.abs(p - st.pos).max() <= F64_TOL * np.abs(st.pos).max()
        assert np.abs(rho[o:o + n] - st.rho).max() <= F64_TOL * np.abs(st.rho).max()
        o += n
    b.close()


def test_batch_of_one_equals_plain_handle(pg):
    w = workloads.dam_break_2d(dx=0.05)
    b = _batch([w], 0)
    s = ParticleSystem(w["config"], w["n"])
    workloads.load_into(s, w)
    b.step(4)
    s.step(4)
    assert np.array_equal(b.get("pos"), s.get("pos"))
    assert np.array_equal(b.get("rho"), s.get("rho"))


def test_batch_overlapped_step_within_tolerance(pg, oracle):
    """A double-word batch of more than 1M particles takes the overlapped schedule (lists of
    the first slots, continuity passes beside the rest of the lists on a second stream); the
    split falls inside a system.  Every system stays within the f64 tolerance of its oracle run."""
    systems = workloads.batched_dam_breaks(n_systems=40, nmin=20000, nmax=40000, seed=12)
    assert sum(w["n"] for w in systems) >= 1000000
    b = _batch(systems, 1)
    split = b.info()["overlap_split"]
    assert 0 < split < b.n
    bounds = np.cumsum([0] + [w["n"] for w in systems])
    assert not np.isin(split, bounds)  # the split is inside a system
    nsteps = 2
    b.step(nsteps)
    ref = _oracle_runs(oracle, systems, nsteps)
    pos, rho = b.get("pos"), b.get("rho")
    o = 0
    for w, st in zip(systems, ref):
        n = w["n"]
        assert np.abs(pos[o:o + n] - st.pos).max() <= F64_TOL * np.abs(st.pos).max()
        assert np.abs(rho[o:o + n] - st.rho).max() <= F64_TOL * np.abs(st.rho).max()
        o += n
    b.close()


def test_double_word_system_alone_equals_it_in_a_batch(pg):
    """The double-word packs are shifted per system, so a system's bits do not depend on the
    other systems of its batch: each system stepped alone equals it stepped in the batch."""
    systems = _small_systems(count=5, seed=9)
    b = _batch(systems, 1)
    b.step(4)
    pos, vel, rho = b.get("pos"), b.get("vel"), b.get("rho")
    b.close()
    o = 0
    for w in systems:
        n = w["n"]
        s = ParticleSystem(dict(w["config"], f64_mode=1), n)
        workloads.load_into(s, w)
        s.step(4)
        assert np.array_equal(s.get("pos"), pos[o:o + n])
        assert np.array_equal(s.get("vel"), vel[o:o + n])
        assert np.array_equal(s.get("rho"), rho[o:o + n])
        s.close()
        o += n
