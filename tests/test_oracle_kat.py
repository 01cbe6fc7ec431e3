"""Known-answer tests of the CPU oracle (no GPU).

The reference has no numeric tests and no golden data (its two tests print the equation IR
and the generated loop text), so the oracle is pinned here by answers derived by hand:
  * cell list: the hash formula, a stable sort by cell and the cell table, against numpy;
  * neighbour sets and the eq1 gather (force[i] += mass[j] of the reference's only equation)
    against brute force over all pairs, bit for bit (integer-valued masses sum exactly);
  * SPH continuity: for v = A x on a lattice interior, drho = -rho0 tr(A) to the kernel's
    discretisation error (< 1 %), in 2D and 3D;
  * SPH momentum: uniform motion gives a zero density rate exactly and, at uniform pressure,
    forces that cancel to rounding on the lattice interior; a linear density profile gives
    a = -grad(p)/rho to < 1.5 % and no transverse force;
  * SPH pair forces: on a disordered cloud with viscosity, unequal masses and densities, total
    linear and angular momentum rates vanish to rounding (antisymmetric, central pair terms),
    and rotating the configuration rotates the accelerations (isotropy);
  * DEM: a head-on collision rebounds with the restitution coefficient, and a sphere resting
    on the floor settles at the overlap m g / kn;
  * the dual-number gradient equals central finite differences of the double run.
"""
import math

import numpy as np
import pytest


def lattice(side, dim, dx=0.01):
    n = side ** dim
    idx = np.arange(n)
    cols = [idx % side, (idx // side) % side] + ([idx // (side * side)] if dim == 3 else [])
    return np.stack(cols, 1).astype(np.float64) * dx + 0.5 * dx


def sph_cfg(dim, h, **over):
    c = dict(dim=dim, h=h, rho0=1000.0, c0=10.0, alpha=0.0, eps_av=0.01, tait_B=1000.0 * 100 / 7, gamma=7, dt=1e-5,
             domain_lo=[-0.1] * 3, domain_hi=[0.5] * 3, cell_multiplier=1.0, gravity=[0, 0, 0], n_fluid=-1)
    if dim == 2:
        c["domain_lo"][2] = c["domain_hi"][2] = 0.0
    c.update(over)
    return c


def test_cell_list_matches_numpy(oracle):
    rng = np.random.default_rng(0)
    pos = rng.uniform(-0.05, 1.05, size=(3000, 3))  # some outside the box: clamped into edge cells
    lo, hi, support = [0.0, 0.0, 0.0], [1.0, 1.0, 1.0], 0.07
    cell, sid, start = oracle.cell_list(pos, lo, hi, support)
    g = oracle.grid(3, lo, hi, support, 1.0)
    nx, ny, nz = g["n"]
    side = g["cell"]
    c = np.clip(np.floor((pos - np.array(lo)) * (1.0 / side)), 0, np.array([nx, ny, nz]) - 1).astype(np.int64)
    key = (c[:, 2] * ny + c[:, 1]) * nx + c[:, 0]
    assert np.array_equal(cell, key)
    assert np.array_equal(sid, np.argsort(key, kind="stable"))
    assert np.array_equal(start, np.searchsorted(np.sort(key), np.arange(nx * ny * nz + 1), side="left"))


@pytest.mark.parametrize("dim", [2, 3])
def test_neighbor_sets_and_eq1_match_brute_force(oracle, dim):
    rng = np.random.default_rng(dim)
    n = 700
    pos = rng.uniform(0.0, 0.3, size=(n, dim))
    lo, hi, support = [0.0] * 3, [0.3] * 3, 0.04
    d = pos[:, None, :] - pos[None, :, :]
    r2 = d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]
    if dim == 3:
        r2 = r2 + d[..., 2] * d[..., 2]
    nbr = r2 < support * support
    counts = oracle.neighbor_counts(pos, lo, hi, support)
    assert np.array_equal(counts, nbr.sum(1))
    offs, lst = oracle.neighbor_list(pos, lo, hi, support)
    for i in range(0, n, 37):
        assert sorted(lst[offs[i]:offs[i + 1]]) == list(np.nonzero(nbr[i])[0])
    mass = rng.integers(1, 1000, size=n).astype(np.float64)
    force = rng.integers(-50, 50, size=n).astype(np.float64)
    out = oracle.gather_sum(pos, lo, hi, support, mass, force)
    assert np.array_equal(out, force + nbr.astype(np.float64) @ mass)


@pytest.mark.parametrize("dim,side,hfac,A", [
    (3, 20, 1.3, [[0.3, 0.1, 0.0], [0.0, -0.2, 0.05], [0.1, 0.0, 0.4]]),
    (2, 40, 1.2, [[0.5, 0.1], [0.2, -0.1]]),
])
def test_continuity_of_a_linear_velocity_field(oracle, dim, side, hfac, A):
    dx = 0.01
    A = np.array(A)
    pos = lattice(side, dim, dx)
    n = pos.shape[0]
    h = hfac * dx
    st = oracle.SphState(pos, pos @ A.T, np.full(n, 1000.0), np.full(n, 1000.0 * dx ** dim))
    _, drho = oracle.sph_rates(sph_cfg(dim, h), st)
    interior = np.all((pos > 4 * h) & (pos < side * dx - 4 * h), axis=1)
    ratio = drho[interior] / (-1000.0 * np.trace(A))
    assert np.all(np.abs(ratio - 1.0) < 0.01)


def test_uniform_motion_has_zero_rates(oracle):
    dx = 0.01
    pos = lattice(16, 3, dx)
    n = pos.shape[0]
    st = oracle.SphState(pos, np.tile([0.1, 0.2, -0.3], (n, 1)), np.full(n, 1003.0), np.full(n, 1e-3))
    acc, drho = oracle.sph_rates(sph_cfg(3, 1.3 * dx, alpha=0.1), st)
    interior = np.all((pos > 0.04) & (pos < 0.12), axis=1)
    assert np.all(drho == 0.0)
    # pair terms are about m 2P F r ~ 10 m/s^2; their sum cancels to rounding
    assert np.abs(acc[interior]).max() < 1e-10


def test_pressure_gradient_force(oracle):
    dx = 0.01
    pos = lattice(20, 3, dx)
    n = pos.shape[0]
    beta = 0.01
    rho = 1000.0 * (1.0 + beta * pos[:, 2])
    cfg = sph_cfg(3, 1.3 * dx)
    st = oracle.SphState(pos, np.zeros_like(pos), rho, np.full(n, 1e-3))
    acc, _ = oracle.sph_rates(cfg, st)
    B = cfg["tait_B"]
    dpdz = B * 7 * (rho / 1000.0) ** 6 * beta
    pred = -dpdz / rho
    interior = np.all((pos > 4 * 1.3 * dx) & (pos < 0.2 - 4 * 1.3 * dx), axis=1)
    assert np.all(np.abs(acc[interior, 2] / pred[interior] - 1.0) < 0.015)
    assert np.abs(acc[interior, :2]).max() < 1e-9 * np.abs(pred).max()


def _dem_cfg(r, **over):
    c = dict(kn=1e5, restitution=0.9, mu=0.3, kt=0.0, dt=1e-7, r_max=r, cell_multiplier=1.0, gravity=[0, 0, 0],
             domain_lo=[0, 0, 0], domain_hi=[0.02] * 3, wall_lo=[-1, -1, -1], wall_hi=[1, 1, 1],
             contact_capacity=4)
    c.update(over)
    return c


def test_dem_head_on_restitution(oracle):
    r = 0.5e-3
    m = 2600 * 4 / 3 * math.pi * r ** 3
    pos = np.array([[0.01 - 1.05 * r, 0.01, 0.01], [0.01 + 1.05 * r, 0.01, 0.01]])
    vel = np.array([[0.1, 0, 0], [-0.1, 0, 0]])
    st = oracle.DemState(pos, vel, np.zeros((2, 3)), np.full(2, r), np.full(2, m), 4)
    oracle.dem_run(_dem_cfg(r), st, 4000)
    v = st.vel
    assert abs((v[1, 0] - v[0, 0]) / 0.2 - 0.9) < 0.005
    assert np.all(v[:, 1:] == 0.0) and np.all(st.omega == 0.0)


def test_dem_sphere_rests_at_static_overlap(oracle):
    r = 0.5e-3
    m = 2600 * 4 / 3 * math.pi * r ** 3
    cfg = _dem_cfg(r, gravity=[0, 0, -9.81], wall_lo=[0, 0, 0], wall_hi=[0.02] * 3, dt=1e-6, restitution=0.3)
    st = oracle.DemState(np.array([[0.01, 0.01, r]]), np.zeros((1, 3)), np.zeros((1, 3)), np.full(1, r),
                         np.full(1, m), 4)
    oracle.dem_run(cfg, st, 200000)
    overlap = r - st.pos[0, 2]
    assert abs(overlap / (m * 9.81 / 1e5) - 1.0) < 1e-6


def test_dual_number_gradient_matches_finite_differences(oracle):
    from prestige_gb300 import workloads
    w = workloads.differentiable_3d(n=512, seed=4, target_seed=5)
    cfg = w["config"]
    f = w["fields"]
    nsteps = 6

    def loss(**over):
        c = dict(cfg, **over)
        st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
        oracle.sph_run(c, st, nsteps)
        e = st.pos - w["target"]
        return float((e * e).sum() / w["n"])

    st = oracle.SphState(f["pos"], f["vel"], f["rho"], f["mass"])
    u = np.zeros_like(f["vel"])
    L, da, dB, _ = oracle.sph_grad_dual(cfg, st, u, w["target"], nsteps)
    assert abs(L - loss()) <= 1e-14 * abs(L)
    # central differences at eps = 1e-6 carry about 1e-16 L / eps of rounding, ~1e-6 relative here
    ea = 1e-6
    fd_a = (loss(alpha=cfg["alpha"] + ea) - loss(alpha=cfg["alpha"] - ea)) / (2 * ea)
    assert abs(da - fd_a) <= 1e-5 * abs(fd_a)
    # dL/dB is ~1e-16 after 6 steps; a relative step of 1e-4 keeps the rounding below 1e-5
    eb = 1e-4 * cfg["tait_B"]
    fd_b = (loss(tait_B=cfg["tait_B"] + eb) - loss(tait_B=cfg["tait_B"] - eb)) / (2 * eb)
    assert abs(dB - fd_b) <= 1e-5 * abs(fd_b)


def test_oracle_states_do_not_alias_inputs(oracle):
    """The oracle advances its state in place; the caller's arrays must stay untouched."""
    from prestige_gb300 import workloads
    w = workloads.sph_lattice_3d(n=300, seed=3)
    f = {k: v.copy() for k, v in w["fields"].items()}
    st = oracle.SphState(w["fields"]["pos"], w["fields"]["vel"], w["fields"]["rho"], w["fields"]["mass"])
    oracle.sph_run(w["config"], st, 2)
    for k in f:
        assert np.array_equal(f[k], w["fields"][k])


def _random_cloud(dim, n=1500, seed=3, dx=0.01):
    """A disordered cloud (a jittered lattice, random velocities and densities) in free space."""
    rng = np.random.default_rng(seed)
    side = int(round(n ** (1.0 / dim)))
    pos = lattice(side, dim, dx) + rng.uniform(-0.3 * dx, 0.3 * dx, size=(side ** dim, dim))
    m = pos.shape[0]
    vel = rng.normal(0.0, 0.5, size=pos.shape)
    rho = 1000.0 * (1.0 + rng.uniform(-0.02, 0.02, size=m))
    mass = 1000.0 * dx ** dim * (1.0 + rng.uniform(-0.1, 0.1, size=m))
    return pos, vel, rho, mass


@pytest.mark.parametrize("dim", [2, 3])
def test_pair_forces_conserve_momentum(oracle, dim):
    """Every pair term is antisymmetric (the symmetric factor (P_i + P_j + Pi_ij) F_ij times
    x_ij = -x_ji, weighted by the partner's mass), so sum_i m_i a_i vanishes to rounding, with
    viscosity on and unequal masses and densities."""
    dx = 0.01
    pos, vel, rho, mass = _random_cloud(dim, dx=dx)
    cfg = sph_cfg(dim, 1.3 * dx, alpha=0.3)
    acc, _ = oracle.sph_rates(cfg, oracle.SphState(pos, vel, rho, mass))
    total = (mass[:, None] * acc).sum(axis=0)
    scale = np.abs(mass[:, None] * acc).sum(axis=0)
    assert np.all(np.abs(total) <= 1e-12 * scale)


def test_pair_forces_conserve_angular_momentum(oracle):
    """The pair forces act along x_ij, so sum_i m_i x_i x a_i vanishes to rounding (3D)."""
    dx = 0.01
    pos, vel, rho, mass = _random_cloud(3, dx=dx)
    acc, _ = oracle.sph_rates(sph_cfg(3, 1.3 * dx, alpha=0.3), oracle.SphState(pos, vel, rho, mass))
    torque = np.cross(pos, mass[:, None] * acc)
    assert np.all(np.abs(torque.sum(axis=0)) <= 1e-12 * np.abs(torque).sum(axis=0))


def test_rates_rotate_with_the_configuration(oracle):
    """Rotating positions and velocities rotates the accelerations and leaves the density rates
    unchanged (the method has no preferred direction; the cell grid only orders the sums)."""
    dx = 0.01
    pos, vel, rho, mass = _random_cloud(3, n=1200, dx=dx)
    cfg = sph_cfg(3, 1.3 * dx, alpha=0.3)
    a0, d0 = oracle.sph_rates(cfg, oracle.SphState(pos, vel, rho, mass))
    q, _ = np.linalg.qr(np.random.default_rng(8).normal(size=(3, 3)))
    centre = pos.mean(axis=0)
    pos_r = (pos - centre) @ q.T + 0.25
    a1, d1 = oracle.sph_rates(cfg, oracle.SphState(pos_r, vel @ q.T, rho, mass))
    scale = np.abs(a0).max()
    assert np.abs(a1 - a0 @ q.T).max() <= 1e-9 * scale
    assert np.abs(d1 - d0).max() <= 1e-9 * np.abs(d0).max()
