"""Adjoint of the SPH step on the GPU (pg_forward_checkpointed + pg_backward).

Checks
  * against central finite differences of the GPU forward run (IEEE f64 mode): relative
    agreement 1e-5 for dL/dalpha, dL/dB and sampled components of dL/dv0, for the FP64 adjoint
    (IEEE handles) and the mixed-precision adjoint (fast f64 handles);
  * against the oracle's forward-mode dual-number gradient (same loss, same steps): relative
    1e-8 for the FP64 adjoint and 1e-5 for the mixed-precision one, for dL/dalpha, dL/dB and
    the directional derivative <dL/dv0, u>;
  * the checkpoint interval does not change the result (bit for bit for the double-word handle;
    within 1e-11 for the IEEE handle, whose segments are recomputed in the double-word mode), the
    handle's state after pg_backward is the final forward state, and the handle steps in its own
    mode and schedule afterwards.
Loss: L = mean over fluid particles of |x_i(T) - target_i|^2, so dL/dx_i = 2 (x_i - t_i) / n_fluid.
"""
import numpy as np
import pytest

from prestige_gb300 import ParticleSystem, make_config, workloads

pytestmark = pytest.mark.gpu

FD_TOL = 1e-5
DUAL_TOL = 1e-8


def _system(w, **over):
    cfg = dict(w["config"])
    cfg.update(over)
    s = ParticleSystem(make_config(**cfg), w["n"])
    workloads.load_into(s, w)
    return s, cfg


def _nfluid(w):
    return w.get("n_fluid", w["n"])


def _loss(w, x):
    nf = _nfluid(w)
    e = x[:nf] - w["target"][:nf]
    return float((e * e).sum() / nf)


def _dloss(w, x):
    nf = _nfluid(w)
    g = np.zeros_like(x)
    g[:nf] = 2.0 * (x[:nf] - w["target"][:nf]) / nf
    return g


def _forward_loss(w, nsteps, vel=None, **over):
    s, _ = _system(w, **over)
    if vel is not None:
        s.set("vel", vel)
    s.step(nsteps)
    L = _loss(w, s.get("pos"))
    s.close()
    return L


def _gradients(w, nsteps, every, **over):
    s, cfg = _system(w, **over)
    s.forward_checkpointed(nsteps, every)
    xT = s.get("pos")
    da, dB, dv0 = s.backward(_dloss(w, xT))
    after = s.get("pos")
    s.close()
    return da, dB, dv0, xT, after, cfg


def _small_3d():
    w = workloads.differentiable_3d(n=1728, seed=4, target_seed=5)
    return w


@pytest.mark.parametrize("mode", [0, 1])
def test_adjoint_matches_finite_differences(pg, mode):
    w = _small_3d()
    nsteps, every = 12, 5
    da, dB, dv0, xT, after, cfg = _gradients(w, nsteps, every, f64_mode=mode)
    assert np.array_equal(xT, after)
    # finite differences below run the IEEE forward (_forward_loss keeps the workload's mode 0)
    # dL/dalpha
    ea = 1e-6
    fd_a = (_forward_loss(w, nsteps, alpha=cfg["alpha"] + ea) - _forward_loss(w, nsteps, alpha=cfg["alpha"] - ea)) / (
        2 * ea)
    assert abs(da - fd_a) <= FD_TOL * abs(fd_a), (da, fd_a)
    # dL/dB (relative step)
    B = cfg["tait_B"]
    eb = 1e-6 * B
    fd_b = (_forward_loss(w, nsteps, tait_B=B + eb) - _forward_loss(w, nsteps, tait_B=B - eb)) / (2 * eb)
    assert abs(dB - fd_b) <= FD_TOL * abs(fd_b), (dB, fd_b)
    # a few initial-velocity components, the largest first
    rng = np.random.default_rng(0)
    flat = np.abs(dv0).ravel()
    picks = [int(np.argmax(flat))] + list(rng.choice(flat.size, 3, replace=False))
    v0 = w["fields"]["vel"]
    ev = 1e-6
    for p in picks:
        i, c = divmod(p, 3)
        vp = v0.copy()
        vm = v0.copy()
        vp[i, c] += ev
        vm[i, c] -= ev
        fd = (_forward_loss(w, nsteps, vel=vp) - _forward_loss(w, nsteps, vel=vm)) / (2 * ev)
        # components far below the largest are compared against a floor of the norm: 1e-3 of
        # the largest for the FP64 adjoint, 1e-2 for the mixed-precision one (FP32 pair terms:
        # measured within 4e-6 of the FP64 adjoint on components above 1e-2 of the largest,
        # within 3e-5 above 1e-3)
        scale = max(abs(fd), (1e-3 if mode == 0 else 1e-2) * flat.max())
        assert abs(dv0[i, c] - fd) <= FD_TOL * scale, (i, c, dv0[i, c], fd)


def _dual_check(oracle, w, nsteps, every, mode=0, **over):
    da, dB, dv0, _, _, cfg = _gradients(w, nsteps, every, f64_mode=mode, **over)
    tol = DUAL_TOL if mode == 0 else FD_TOL
    rng = np.random.default_rng(7)
    u = rng.normal(size=w["fields"]["vel"].shape)
    f = w["fields"]
    st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    L, oa, ob, ou = oracle.sph_grad_dual(cfg, st, u, w["target"], nsteps)
    jvp = float((dv0 * u).sum())
    assert abs(da - oa) <= tol * abs(oa), (da, oa)
    assert abs(dB - ob) <= tol * abs(ob), (dB, ob)
    assert abs(jvp - ou) <= tol * abs(ou), (jvp, ou)


@pytest.mark.parametrize("mode", [0, 1])
def test_adjoint_matches_dual_number_oracle_3d(pg, oracle, mode):
    _dual_check(oracle, _small_3d(), nsteps=20, every=6, mode=mode)


@pytest.mark.parametrize("mode", [0, 1])
def test_adjoint_matches_dual_number_oracle_2d_walls(pg, oracle, mode):
    w = workloads.dam_break_2d(dx=0.05)
    rng = np.random.default_rng(11)
    w["fields"]["vel"] = rng.normal(0.0, 0.05, size=w["fields"]["pos"].shape)
    w["fields"]["vel"][w["n_fluid"]:] = 0.0
    w["target"] = w["fields"]["pos"] + rng.normal(0.0, 0.002, size=w["fields"]["pos"].shape)
    _dual_check(oracle, w, nsteps=15, every=4, mode=mode)


@pytest.mark.parametrize("cap", [16, 48])
@pytest.mark.parametrize("mode", [0, 1])
def test_adjoint_with_lists_cut_short_matches_dual_numbers(pg, oracle, mode, cap):
    """Neighbour lists shorter than the neighbour count: the FP64 adjoint's pairs that only one
    list holds are evaluated by each side for itself, and the rest of each list's walk likewise
    (16 entries cut every list among the lower slots, 48 among the upper ones); the mixed adjoint
    follows its lists' continued walks.  The gradients stay within the dual-number bars."""
    _dual_check(oracle, _small_3d(), nsteps=8, every=3, mode=mode, list_capacity=cap)


@pytest.mark.parametrize("mode", [0, 1])
def test_checkpoint_interval_does_not_change_gradients(pg, mode):
    """The double-word handle recomputes its segments in its own mode, so the checkpoint interval
    changes nothing, bit for bit.  The IEEE handle recomputes each segment in the double-word
    mode from the segment's IEEE checkpoint, so the states it linearises about depend on where
    the segment starts, within the double-word drift (about 1e-12): the gradients agree to 1e-11."""
    w = _small_3d()
    ref = _gradients(w, 9, 9, f64_mode=mode)
    for every in (1, 4):
        got = _gradients(w, 9, every, f64_mode=mode)
        if mode == 1:
            assert got[0] == ref[0] and got[1] == ref[1]
            assert np.array_equal(got[2], ref[2])
        else:
            assert abs(got[0] - ref[0]) <= 1e-11 * abs(ref[0])
            assert abs(got[1] - ref[1]) <= 1e-11 * abs(ref[1])
            assert np.abs(got[2] - ref[2]).max() <= 1e-11 * np.abs(ref[2]).max()


def test_backward_restores_the_handle(pg):
    """pg_backward on an IEEE handle switches to the double-word mode for its recompute and back:
    afterwards the handle steps in the IEEE mode with its block sizes and graph, bit for bit as
    a handle that never ran the backward pass."""
    w = _small_3d()
    a, _ = _system(w)
    a.set_momentum_block(128)
    a.enable_graph(True)
    a.forward_checkpointed(4, 2)
    x = a.get("pos")
    a.backward(_dloss(w, x))
    info = a.info()
    assert info["arith"] == 0 and info["momentum_block"] == 128
    b, _ = _system(w)
    b.step(4)
    a.step(3)
    b.step(3)
    assert np.array_equal(a.get("pos"), b.get("pos")) and np.array_equal(a.get("rho"), b.get("rho"))
    a.close()
    b.close()


def test_backward_needs_forward(pg):
    w = _small_3d()
    s, _ = _system(w)
    with pytest.raises(Exception):
        s.backward(np.zeros((w["n"], 3)))
    s.close()
