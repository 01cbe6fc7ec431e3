"""The adjoint at the size of the differentiable workload: 100,000 particles, 500 steps,
checkpoints every 50 (ten recomputed segments), and at 10,000 particles over two segments.

References
  * the oracle's forward-mode dual-number run of the same loss (dL/dalpha, dL/dB and the
    directional derivative <dL/dv0, u> for a seeded direction u): the FP64 adjoint (IEEE handles)
    agrees to 1e-8 (measured on a GB300: 6e-15, 3e-14 and 1e-14 at full size), the
    mixed-precision adjoint (double-word handles) to 1e-5 for dL/dalpha and <dL/dv0, u>
    (measured 1.3e-7 and 2.7e-8) and to 5e-5 for dL/dB (measured 1.3e-5 to 1.7e-5: its pair
    terms are about 1e3 times its total, which amplifies the FP32 floor of the pair
    derivatives);
  * central finite differences of the IEEE forward run: dL/dalpha at eps = 1e-6 to 1e-5 for both
    adjoints.  For dL/dB the finite difference itself is the less accurate side at this size: the
    artificial viscosity switches on where v_ij . x_ij changes sign, a kink that some of the
    3.7e9 pair evaluations of the run cross inside the difference interval, so the difference
    quotient's error falls with eps (measured against the dual-number value: 3.4e-3, 6.4e-4,
    4.7e-5, 1.5e-5 at relative eps 1e-4 ... 1e-7) while the adjoint matches the dual-number value
    to 3e-14.  The test checks that convergence: the quotient approaches the adjoint as eps falls
    and is within 5e-5 of it at eps = 1e-7.
Loss: L = mean over particles of |x_i(T) - target_i|^2.
"""
import numpy as np
import pytest

from prestige_gb300 import ParticleSystem, make_config, workloads

pytestmark = pytest.mark.gpu

N_FULL, STEPS_FULL, EVERY_FULL = 100000, 500, 50


def _system(w, **over):
    cfg = dict(w["config"])
    cfg.update(over)
    s = ParticleSystem(make_config(**cfg), w["n"])
    workloads.load_into(s, w)
    return s, cfg


def _loss(w, x):
    e = x - w["target"]
    return float((e * e).sum() / w["n"])


def _forward_loss(w, nsteps, **over):
    s, _ = _system(w, **over)
    s.step(nsteps)
    L = _loss(w, s.get("pos"))
    s.close()
    return L


def _gradients(w, nsteps, every, mode):
    s, cfg = _system(w, f64_mode=mode)
    s.forward_checkpointed(nsteps, every)
    x = s.get("pos")
    da, dB, dv0 = s.backward(2.0 * (x - w["target"]) / w["n"])
    s.close()
    return da, dB, dv0, cfg


def _dual(oracle, w, nsteps):
    u = np.random.default_rng(7).normal(size=w["fields"]["vel"].shape)
    f = w["fields"]
    st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    L, da, dB, du = oracle.sph_grad_dual(w["config"], st, u, w["target"], nsteps)
    return u, da, dB, du


@pytest.fixture(scope="module")
def full(oracle):
    w = workloads.differentiable_3d(n=N_FULL)
    return w, _dual(oracle, w, STEPS_FULL)


def _rel(a, b):
    return abs(a - b) / abs(b)


@pytest.mark.parametrize("mode", [0, 1])
def test_two_segments_at_10k_against_dual_numbers(pg, oracle, mode):
    w = workloads.differentiable_3d(n=10000)
    u, oa, ob, ou = _dual(oracle, w, 100)
    da, dB, dv0, _ = _gradients(w, 100, 50, mode)
    tol = 1e-8 if mode == 0 else 1e-5
    assert _rel(da, oa) <= tol
    assert _rel(dB, ob) <= tol
    assert _rel(float((dv0 * u).sum()), ou) <= tol


@pytest.mark.parametrize("mode", [0, 1])
def test_full_size_against_dual_numbers(pg, full, mode):
    w, (u, oa, ob, ou) = full
    da, dB, dv0, _ = _gradients(w, STEPS_FULL, EVERY_FULL, mode)
    if mode == 0:
        assert _rel(da, oa) <= 1e-8 and _rel(dB, ob) <= 1e-8
        assert _rel(float((dv0 * u).sum()), ou) <= 1e-8
    else:
        assert _rel(da, oa) <= 1e-5
        assert _rel(float((dv0 * u).sum()), ou) <= 1e-5
        assert _rel(dB, ob) <= 5e-5


def test_full_size_mixed_initial_velocity_components(pg, full):
    """dL/dv0 component by component: the mixed-precision adjoint against the FP64 one (which
    matches the dual-number oracle to 1e-14): within 1e-5 on components above 1e-2 of the largest
    and 1e-4 above 1e-3 (measured 3.9e-6 and 2.4e-5)."""
    w, _ = full
    g0 = _gradients(w, STEPS_FULL, EVERY_FULL, 0)[2]
    g1 = _gradients(w, STEPS_FULL, EVERY_FULL, 1)[2]
    mx = np.abs(g0).max()
    for floor, tol in ((1e-2, 1e-5), (1e-3, 1e-4)):
        sel = np.abs(g0) >= floor * mx
        assert (np.abs(g1 - g0)[sel] / np.abs(g0)[sel]).max() <= tol


@pytest.mark.parametrize("mode", [0, 1])
def test_full_size_alpha_against_finite_differences(pg, full, mode):
    w, _ = full
    da, _, _, cfg = _gradients(w, STEPS_FULL, EVERY_FULL, mode)
    ea = 1e-6
    fd = (_forward_loss(w, STEPS_FULL, alpha=cfg["alpha"] + ea) -
          _forward_loss(w, STEPS_FULL, alpha=cfg["alpha"] - ea)) / (2 * ea)
    assert _rel(da, fd) <= 1e-5


def test_full_size_tait_b_finite_differences_converge_to_the_adjoint(pg, full):
    w, _ = full
    _, dB, _, cfg = _gradients(w, STEPS_FULL, EVERY_FULL, 0)
    B = cfg["tait_B"]
    errs = []
    for rel_eps in (1e-5, 1e-7):
        eb = rel_eps * B
        fd = (_forward_loss(w, STEPS_FULL, tait_B=B + eb) - _forward_loss(w, STEPS_FULL, tait_B=B - eb)) / (2 * eb)
        errs.append(_rel(fd, dB))
    assert errs[1] < errs[0]
    assert errs[1] <= 5e-5
