"""Asynchronous host I/O (pg_set_field_async / pg_get_field_async / pg_wait_io).

A step loop that feeds inputs and reads results through the asynchronous calls must give the
same numbers, bit for bit, as the same loop through pg_set_field / pg_step / pg_get_field: the
copies only move in time.  Ordering rules checked here: a staged input takes effect before the
next call on the handle (a later synchronous set wins over it, a read sees it); a snapshot taken
before a step holds the pre-step values after the step.
"""
import numpy as np
import pytest

from prestige_gb300 import ParticleSystem, make_config, workloads
from prestige_gb300 import _native as nat

pytestmark = pytest.mark.gpu

FIELDS_IN = ("pos", "vel", "rho", "mass")
FIELDS_OUT = ("pos", "vel", "rho")


def _system(w, f64_mode):
    cfg = dict(w["config"])
    cfg.update(precision=1, f64_mode=f64_mode)
    s = ParticleSystem(make_config(**cfg), w["n"])
    for k in FIELDS_IN:
        s.set(k, np.asarray(w["fields"][k], np.float64))
    return s


def _pinned(a):
    torch = pytest.importorskip("torch")
    t = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
    t.numpy()[:] = np.asarray(a, np.float64).reshape(-1)
    return t


def _inputs(w, steps):
    """Per-step inputs: the workload state perturbed differently every step."""
    rng = np.random.default_rng(11)
    out = []
    for _ in range(steps):
        f = {k: np.asarray(w["fields"][k], np.float64).copy() for k in FIELDS_IN}
        f["vel"] = f["vel"] + rng.normal(0.0, 0.01, size=f["vel"].shape)
        f["rho"] = f["rho"] * (1.0 + rng.uniform(-1e-3, 1e-3, size=f["rho"].shape))
        out.append(f)
    return out


@pytest.mark.parametrize("f64_mode", [0, 1])
def test_async_loop_matches_sync_loop(pg, f64_mode):
    w = workloads.sph_lattice_3d(n=20000, seed=5)
    steps = 4
    ins = _inputs(w, steps)

    s = _system(w, f64_mode)
    ref = []
    for f in ins:
        for k in FIELDS_IN:
            s.set(k, f[k])
        s.step(1)
        ref.append({k: s.get(k).reshape(-1).copy() for k in FIELDS_OUT})
    s.close()

    s = _system(w, f64_mode)
    pin_in = [{k: _pinned(f[k]) for k in FIELDS_IN} for f in ins]
    pin_out = [{k: _pinned(np.zeros_like(ref[0][k])) for k in FIELDS_OUT} for _ in range(steps)]
    for i in range(steps):
        for k in FIELDS_IN:
            s.set_ptr_async(k, pin_in[i][k].data_ptr(), pin_in[i][k].numel())
        s.step_async(1)
        for k in FIELDS_OUT:
            s.get_ptr_async(k, pin_out[i][k].data_ptr(), pin_out[i][k].numel())
    s.wait_io()
    for i in range(steps):
        for k in FIELDS_OUT:
            assert np.array_equal(pin_out[i][k].numpy(), ref[i][k]), (i, k)
    s.close()


def test_staged_input_takes_effect_before_the_next_call(pg):
    w = workloads.sph_lattice_3d(n=2000, seed=6)
    s = _system(w, 1)
    rho = np.asarray(w["fields"]["rho"], np.float64)
    a = _pinned(rho * 1.01)
    s.set_ptr_async("rho", a.data_ptr(), a.numel())
    assert np.array_equal(s.get("rho"), rho * 1.01)  # a read sees the staged value
    b = _pinned(rho * 1.02)
    s.set_ptr_async("rho", b.data_ptr(), b.numel())
    s.set("rho", rho * 1.03)  # a later synchronous set wins
    assert np.array_equal(s.get("rho"), rho * 1.03)
    c1, c2 = _pinned(rho * 1.04), _pinned(rho * 1.05)
    s.set_ptr_async("rho", c1.data_ptr(), c1.numel())
    s.set_ptr_async("rho", c2.data_ptr(), c2.numel())  # the last staged value wins
    s.wait_io()
    assert np.array_equal(s.get("rho"), rho * 1.05)
    s.close()


def test_snapshot_holds_pre_step_values(pg):
    w = workloads.sph_lattice_3d(n=3000, seed=7)
    s = _system(w, 1)
    before = s.get("pos").reshape(-1).copy()
    out = _pinned(np.zeros_like(before))
    s.get_ptr_async("pos", out.data_ptr(), out.numel())
    s.step_async(3)
    s.wait_io()
    assert np.array_equal(out.numpy(), before)
    assert not np.array_equal(s.get("pos").reshape(-1), before)
    s.close()


def test_async_io_errors(pg):
    w = workloads.sph_lattice_3d(n=500, seed=8)
    s = _system(w, 1)
    n = w["n"]
    buf = _pinned(np.zeros(3 * n))
    lib, h = s._lib, s._h
    assert lib.pg_set_field_async(h, b"pos", buf.data_ptr(), 3 * n, nat.PG_F32) == nat.PG_EINVAL  # precision
    assert lib.pg_set_field_async(h, b"pos", buf.data_ptr(), 3 * n - 1, nat.PG_F64) == nat.PG_EINVAL  # count
    assert lib.pg_set_field_async(h, b"nosuch", buf.data_ptr(), n, nat.PG_F64) == nat.PG_ENOTFOUND
    assert lib.pg_get_field_async(h, b"nosuch", buf.data_ptr(), n, nat.PG_F64) == nat.PG_ENOTFOUND
    s.compute_rates()
    assert lib.pg_set_field_async(h, b"acc", buf.data_ptr(), 3 * n, nat.PG_F64) == nat.PG_EINVAL  # read-only
    assert lib.pg_get_field_async(h, b"acc", buf.data_ptr(), 3 * n, nat.PG_F64) == nat.PG_OK
    s.wait_io()
    assert np.array_equal(buf.numpy().reshape(n, 3), s.get("acc"))
    s.close()


def test_async_loop_with_graph_replay(pg):
    """Staged inputs are moved in before a replayed step graph, snapshots taken after it."""
    w = workloads.sph_lattice_3d(n=8000, seed=9)
    ins = _inputs(w, 3)
    s = _system(w, 1)
    ref = []
    for f in ins:
        for k in FIELDS_IN:
            s.set(k, f[k])
        s.step(1)
        ref.append(s.get("rho").copy())
    s.close()
    s = _system(w, 1)
    s.enable_graph(True)
    pin_in = [{k: _pinned(f[k]) for k in FIELDS_IN} for f in ins]
    outs = [_pinned(np.zeros(w["n"])) for _ in ins]
    for i in range(len(ins)):
        for k in FIELDS_IN:
            s.set_ptr_async(k, pin_in[i][k].data_ptr(), pin_in[i][k].numel())
        s.step_async(1)
        s.get_ptr_async("rho", outs[i].data_ptr(), outs[i].numel())
    s.wait_io()
    for i in range(len(ins)):
        assert np.array_equal(outs[i].numpy(), ref[i])
    s.close()
