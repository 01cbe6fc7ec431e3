"""Seeded synthetic inputs for the particle workloads (no datasets are involved).

Every generator returns a dict with
    "config": keyword overrides for make_config(),  "n": particle count,
    "fields": {name: array in id order},            plus workload-specific extras.

Workloads (sizes as named by the project's benchmark list):
  dam_break_2d      2D weakly-compressible SPH dam break: 1.0 x 2.0 m fluid block on a square
                    lattice (dx = 0.02 -> 5,000 particles) in a 4.0 x 3.0 m tank with 3 layers of
                    fixed dummy wall particles; cubic spline h = 1.2 dx; Tait rho0 = 1000,
                    c0 = 10 sqrt(2 g H), gamma = 7; alpha = 0.1; dt = 0.25 h / c0.
  dem_settling      3D DEM: spheres with radii U[0.5, 1.0] mm, density 2600, placed without
                    overlap by seeded random sequential insertion in a 0.1 x 0.1 x 0.3 m box;
                    kn = 1e5, e = 0.9, mu = 0.3, kt = 2/7 kn (assumed), dt = 1e-6.
  sph_lattice_3d    3D SPH on a jittered cubic lattice, dx = 0.01, jitter U(+-0.2 dx),
                    h = 1.3 dx, v ~ N(0, 0.1), rho = 1000 (1 + U(-0.01, 0.01)); c0 = 10 m/s and
                    dt = 0.25 h / c0 are this project's choices (the workload names neither).
  batched_dam_breaks  512 independent 2D dam breaks, N_i log-uniform in [500, 50000], column
                    height H_i ~ U[0.5, 2.0], W_i = H_i / 2, dx_i = sqrt(W_i H_i / N_i), tank scaled
                    by H_i / 2 (the fixed 4 x 3 m tank cannot hold 50,000 particles at dx = 0.02).
  differentiable_3d 3D SPH lattice as sph_lattice_3d with an initial velocity field made of 8
                    seeded Fourier modes of amplitude 0.05 m/s and a seeded target configuration.
"""
import math

import numpy as np

G = 9.81


# ------------------------------------------------------------------------------------------
# 2D dam break
# ------------------------------------------------------------------------------------------
def dam_break_2d(dx=0.02, width=1.0, height=2.0, tank=(4.0, 3.0), layers=3, alpha=0.1, seed=0,
                 precision=1, f64_mode=0, hydrostatic=True):
    nx, ny = int(round(width / dx)), int(round(height / dx))
    ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    fluid = np.stack([(ii.ravel() + 0.5) * dx, (jj.ravel() + 0.5) * dx], axis=1)
    walls = []
    tw, th = tank
    ncol = int(round(tw / dx))
    nrow = int(round(th / dx))
    for L in range(layers):  # bottom, spanning under the side walls
        y = -(L + 0.5) * dx
        xs = (np.arange(-layers, ncol + layers) + 0.5) * dx
        walls.append(np.stack([xs, np.full_like(xs, y)], axis=1))
    for L in range(layers):  # left and right
        ys = (np.arange(nrow) + 0.5) * dx
        walls.append(np.stack([np.full_like(ys, -(L + 0.5) * dx), ys], axis=1))
        walls.append(np.stack([np.full_like(ys, tw + (L + 0.5) * dx), ys], axis=1))
    walls = np.concatenate(walls, axis=0)
    pos = np.concatenate([fluid, walls], axis=0)
    n_fluid = fluid.shape[0]
    n = pos.shape[0]
    rho0 = 1000.0
    h = 1.2 * dx
    c0 = 10.0 * math.sqrt(2.0 * G * height)
    gamma = 7
    B = rho0 * c0 * c0 / gamma
    rho = np.full(n, rho0)
    if hydrostatic:
        depth = height - fluid[:, 1]
        rho[:n_fluid] = rho0 * (1.0 + rho0 * G * depth / B) ** (1.0 / gamma)
    mass = np.full(n, rho0 * dx * dx)
    pad = 2.0 * h
    cfg = dict(model=0, dim=2, precision=precision, gamma=gamma, n_fluid=n_fluid,
               domain_lo=[-layers * dx - pad, -layers * dx - pad, 0.0],
               domain_hi=[tw + layers * dx + pad, th + pad, 0.0],
               cell_multiplier=1.0, h=h, rho0=rho0, c0=c0, alpha=alpha, eps_av=0.01, tait_B=B,
               gravity=[0.0, -G, 0.0], dt=0.25 * h / c0, f64_mode=f64_mode)
    return {"config": cfg, "n": n, "n_fluid": n_fluid,
            "fields": {"pos": pos, "vel": np.zeros_like(pos), "rho": rho, "mass": mass}}


# ------------------------------------------------------------------------------------------
# 3D jittered lattice (SPH sweep)
# ------------------------------------------------------------------------------------------
def lattice_side(n):
    s = int(round(n ** (1.0 / 3.0)))
    while s ** 3 < n:
        s += 1
    return s


def sph_lattice_3d(n=262144, dx=0.01, seed=2, precision=1, f64_mode=0, c0=10.0, alpha=0.1, cell_multiplier=1.0):
    """Jittered cubic lattice of n particles (a full cube of side round(n^(1/3)) trimmed to n)."""
    rng = np.random.default_rng(seed)
    s = lattice_side(n)
    idx = np.arange(n, dtype=np.int64)
    i, j, k = idx % s, (idx // s) % s, idx // (s * s)
    pos = np.stack([i, j, k], axis=1).astype(np.float64) * dx + 0.5 * dx
    pos += rng.uniform(-0.2 * dx, 0.2 * dx, size=pos.shape)
    vel = rng.normal(0.0, 0.1, size=pos.shape)
    rho0 = 1000.0
    rho = rho0 * (1.0 + rng.uniform(-0.01, 0.01, size=n))
    mass = np.full(n, rho0 * dx ** 3)
    h = 1.3 * dx
    extent = s * dx
    pad = 4.0 * h
    cfg = dict(model=0, dim=3, precision=precision, gamma=7, n_fluid=-1,
               domain_lo=[-pad] * 3, domain_hi=[extent + pad] * 3, cell_multiplier=cell_multiplier,
               h=h, rho0=rho0, c0=c0, alpha=alpha, eps_av=0.01, tait_B=rho0 * c0 * c0 / 7.0,
               gravity=[0.0, 0.0, 0.0], dt=0.25 * h / c0, f64_mode=f64_mode)
    return {"config": cfg, "n": n, "fields": {"pos": pos, "vel": vel, "rho": rho, "mass": mass}}


# ------------------------------------------------------------------------------------------
# DEM: random sequential insertion of non-overlapping spheres
# ------------------------------------------------------------------------------------------
def rsa_spheres(n, box=(0.1, 0.1, 0.3), rmin=0.5e-3, rmax=1.0e-3, seed=1, batch=20000, max_rounds=10000):
    """Random sequential insertion: candidates (position, radius) are drawn in order from one
    seeded stream; a candidate is accepted if it overlaps no earlier accepted sphere and fits in
    the box.  Candidates are tested in batches, with conflicts inside a batch resolved in
    candidate order, which gives the same result as testing them one at a time."""
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(seed)
    box = np.asarray(box, dtype=np.float64)
    placed_x = np.empty((0, 3))
    placed_r = np.empty(0)
    rounds = 0
    while placed_r.size < n:
        rounds += 1
        if rounds > max_rounds:
            raise RuntimeError("random sequential insertion did not reach %d spheres" % n)
        r = rng.uniform(rmin, rmax, size=batch)
        x = rng.uniform(0.0, 1.0, size=(batch, 3)) * (box - 2 * r[:, None]) + r[:, None]
        ok = np.ones(batch, dtype=bool)
        if placed_r.size:
            tree = cKDTree(placed_x)
            cand = tree.query_ball_point(x, r=r + rmax)
            for c in range(batch):
                js = cand[c]
                if js:
                    d = np.linalg.norm(placed_x[js] - x[c], axis=1)
                    if np.any(d < placed_r[js] + r[c]):
                        ok[c] = False
        bt = cKDTree(x)
        pairs = bt.query_pairs(2 * rmax, output_type="ndarray")
        conflicts = {}
        if len(pairs):
            d = np.linalg.norm(x[pairs[:, 0]] - x[pairs[:, 1]], axis=1)
            over = pairs[d < r[pairs[:, 0]] + r[pairs[:, 1]]]
            for a, b in over:
                lo, hi = (a, b) if a < b else (b, a)
                conflicts.setdefault(hi, []).append(lo)
        keep = np.zeros(batch, dtype=bool)
        for c in range(batch):
            if not ok[c]:
                continue
            if c in conflicts and any(keep[p] for p in conflicts[c]):
                continue
            keep[c] = True
        sel = np.nonzero(keep)[0][: n - placed_r.size]
        placed_x = np.concatenate([placed_x, x[sel]])
        placed_r = np.concatenate([placed_r, r[sel]])
    return placed_x, placed_r


def dem_settling(n=200000, box=(0.1, 0.1, 0.3), seed=1, capacity=16, cell_multiplier=1.0, dt=1e-6):
    x, r = rsa_spheres(n, box=box, seed=seed)
    density = 2600.0
    m = density * 4.0 / 3.0 * math.pi * r ** 3
    rmax = 1.0e-3
    pad = 2.0 * rmax
    cfg = dict(model=1, dim=3, precision=1, domain_lo=[-pad] * 3,
               domain_hi=[box[0] + pad, box[1] + pad, box[2] + pad], cell_multiplier=cell_multiplier,
               gravity=[0.0, 0.0, -G], dt=dt, kn=1e5, restitution=0.9, mu=0.3, kt=1e5 * 2.0 / 7.0, r_max=rmax,
               wall_lo=[0.0, 0.0, 0.0], wall_hi=list(box), contact_capacity=capacity)
    return {"config": cfg, "n": n,
            "fields": {"pos": x, "vel": np.zeros_like(x), "omega": np.zeros_like(x), "radius": r, "mass": m}}


def dem_compressed_lattice(nside=(8, 8, 8), r=0.5e-3, overlap=0.02, seed=0, capacity=16):
    """Spheres on a cubic lattice spaced 2r(1 - overlap) with small jitter, random velocities and
    spins, inside walls that touch the outer layer: every contact path (normal, tangential
    history, Coulomb slip, torques, walls) is active from the first step."""
    rng = np.random.default_rng(seed)
    nside = tuple(nside) if hasattr(nside, "__len__") else (nside,) * 3
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
    return {"config": cfg, "n": n, "fields": {"pos": pos, "vel": vel, "omega": omega, "radius": radius,
                                              "mass": mass}}


# ------------------------------------------------------------------------------------------
# Batched dam breaks
# ------------------------------------------------------------------------------------------
def batched_dam_breaks(n_systems=512, nmin=500, nmax=50000, seed=3, precision=1, f64_mode=0, layers=3):
    rng = np.random.default_rng(seed)
    ns = np.round(np.exp(rng.uniform(math.log(nmin), math.log(nmax), size=n_systems))).astype(int)
    hs = rng.uniform(0.5, 2.0, size=n_systems)
    systems = []
    for N, H in zip(ns, hs):
        W = H / 2.0
        dx = math.sqrt(W * H / N)
        scale = H / 2.0
        w = dam_break_2d(dx=dx, width=W, height=H, tank=(4.0 * scale, 3.0 * scale), layers=layers,
                         precision=precision, f64_mode=f64_mode)
        systems.append(w)
    return systems


# ------------------------------------------------------------------------------------------
# Differentiable run
# ------------------------------------------------------------------------------------------
def fourier_velocity(pos, modes=8, amplitude=0.05, seed=4, extent=1.0):
    rng = np.random.default_rng(seed)
    v = np.zeros_like(pos)
    for _ in range(modes):
        kvec = rng.integers(1, 4, size=3) * (2.0 * math.pi / extent) * rng.choice([-1, 1], size=3)
        phase = rng.uniform(0.0, 2.0 * math.pi)
        direction = rng.normal(size=3)
        direction /= np.linalg.norm(direction)
        v += amplitude / modes * np.outer(np.sin(pos @ kvec + phase), direction)
    return v


def differentiable_3d(n=100000, dx=0.01, seed=4, target_seed=5, precision=1):
    w = sph_lattice_3d(n=n, dx=dx, seed=seed, precision=precision)
    pos = w["fields"]["pos"]
    extent = lattice_side(n) * dx
    w["fields"]["vel"] = fourier_velocity(pos, seed=seed, extent=extent)
    w["fields"]["rho"] = np.full(n, 1000.0)
    rng = np.random.default_rng(target_seed)
    w["target"] = pos + rng.normal(0.0, 0.05 * dx, size=pos.shape)
    return w


def load_into(system, w):
    for name, arr in w["fields"].items():
        system.set(name, arr)
    return system
