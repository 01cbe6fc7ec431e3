"""ctypes face of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py, as the reference results the GPU path is compared with or as the timed CPU baseline
-- never by the product library.

The oracle restates the method on the CPU (prestige_oracle.hpp).  Parity with the reference is
unpinned: the reference (dineshadepu/prestige) has no executable numeric path, no numeric tests
and no golden vectors (its codegen returns text, prestige/src/codegen/simple_cpu.rs:3-22).
The oracle is pinned instead by hand-derived known answers (tests/test_oracle_kat.py) and by the
reference's one checkable behaviour, the eq1 gather semantics (prestige/src/lib.rs:7-12).
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build as _build  # noqa: E402

_d3 = ctypes.c_double * 3


class OrcSphSpec(ctypes.Structure):
    _fields_ = [("h", ctypes.c_double), ("rho0", ctypes.c_double), ("c0", ctypes.c_double),
                ("alpha", ctypes.c_double), ("eps", ctypes.c_double), ("B", ctypes.c_double),
                ("dt", ctypes.c_double), ("cell_mult", ctypes.c_double),
                ("g", _d3), ("lo", _d3), ("hi", _d3),
                ("n_fluid", ctypes.c_longlong), ("dim", ctypes.c_int), ("gamma", ctypes.c_int)]


class OrcDemSpec(ctypes.Structure):
    _fields_ = [("kn", ctypes.c_double), ("e", ctypes.c_double), ("mu", ctypes.c_double), ("kt", ctypes.c_double),
                ("dt", ctypes.c_double), ("r_max", ctypes.c_double), ("cell_mult", ctypes.c_double),
                ("g", _d3), ("lo", _d3), ("hi", _d3), ("wall_lo", _d3), ("wall_hi", _d3),
                ("capacity", ctypes.c_int), ("pad", ctypes.c_int)]


_lib = None


def load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build())
        _lib.orc_sph_run.restype = ctypes.c_double
        _lib.orc_grid.restype = ctypes.c_longlong
        _lib.orc_dem_run.restype = ctypes.c_longlong
    return _lib


def _p(a):
    """Host pointer of a numpy array as a ctypes void pointer (a bare Python
    int would be passed as a C int)."""
    return ctypes.c_void_p(a.ctypes.data)


def num_threads(n=0):
    return load().orc_num_threads(int(n))


def _cols(pos, dtype):
    pos = np.asarray(pos)
    dim = pos.shape[1]
    cols = [np.array(pos[:, d], dtype=dtype, copy=True) for d in range(dim)]
    if dim == 2:
        cols.append(np.zeros(pos.shape[0], dtype=dtype))
    return cols


def _d(v):
    a = _d3()
    vv = list(v) + [0.0] * (3 - len(v))
    for i in range(3):
        a[i] = float(vv[i])
    return a


def grid(dim, lo, hi, support, mult):
    n3 = (ctypes.c_int * 3)()
    reach = ctypes.c_int()
    cell = ctypes.c_double()
    nc = load().orc_grid(dim, _d(lo), _d(hi), ctypes.c_double(support), ctypes.c_double(mult), n3,
                         ctypes.byref(reach), ctypes.byref(cell))
    return {"ncells": nc, "n": list(n3), "reach": reach.value, "cell": cell.value}


def cell_list(pos, lo, hi, support, mult=1.0, f64=True):
    dt = np.float64 if f64 else np.float32
    n, dim = np.asarray(pos).shape
    cols = _cols(pos, dt)
    g = grid(dim, lo, hi, support, mult)
    cell = np.empty(n, np.uint32)
    sid = np.empty(n, np.uint32)
    start = np.empty(g["ncells"] + 1, np.uint32)
    load().orc_cell_list(dim, 1 if f64 else 0, ctypes.c_longlong(n), _p(cols[0]), _p(cols[1]),
                         _p(cols[2]), _d(lo), _d(hi), ctypes.c_double(support), ctypes.c_double(mult),
                         _p(cell), _p(sid), _p(start))
    return cell, sid, start


def neighbor_counts(pos, lo, hi, support, mult=1.0, f64=True):
    dt = np.float64 if f64 else np.float32
    n, dim = np.asarray(pos).shape
    cols = _cols(pos, dt)
    out = np.empty(n, np.uint32)
    load().orc_neighbor_counts(dim, 1 if f64 else 0, ctypes.c_longlong(n), _p(cols[0]), _p(cols[1]),
                               _p(cols[2]), _d(lo), _d(hi), ctypes.c_double(support), ctypes.c_double(mult),
                               _p(out))
    return out


def neighbor_list(pos, lo, hi, support, mult=1.0, f64=True):
    dt = np.float64 if f64 else np.float32
    n, dim = np.asarray(pos).shape
    cols = _cols(pos, dt)
    counts = neighbor_counts(pos, lo, hi, support, mult, f64)
    cap = int(counts.sum())
    offs = np.empty(n + 1, np.uint64)
    nbr = np.empty(max(cap, 1), np.uint32)
    st = load().orc_neighbor_list(dim, 1 if f64 else 0, ctypes.c_longlong(n), _p(cols[0]),
                                  _p(cols[1]), _p(cols[2]), _d(lo), _d(hi), ctypes.c_double(support),
                                  ctypes.c_double(mult), _p(offs), _p(nbr), ctypes.c_uint64(cap))
    assert st == 0
    return offs, nbr[:cap]


def gather_sum(pos, lo, hi, support, src, dst, mult=1.0, f64=True):
    dt = np.float64 if f64 else np.float32
    n, dim = np.asarray(pos).shape
    cols = _cols(pos, dt)
    src = np.ascontiguousarray(src, np.float64)
    out = np.array(dst, dtype=np.float64, copy=True)
    load().orc_gather_sum(dim, 1 if f64 else 0, ctypes.c_longlong(n), _p(cols[0]), _p(cols[1]),
                          _p(cols[2]), _d(lo), _d(hi), ctypes.c_double(support), ctypes.c_double(mult),
                          _p(src), _p(out))
    return out


def sph_spec(cfg, n):
    """Oracle spec from a pg_config keyword dict (tait_B must be given explicitly)."""
    s = OrcSphSpec()
    s.h, s.rho0, s.c0, s.alpha = cfg["h"], cfg["rho0"], cfg["c0"], cfg["alpha"]
    s.eps = cfg.get("eps_av", 0.01)
    B = cfg.get("tait_B", 0.0)
    if not B or B <= 0:
        B = cfg["rho0"] * cfg["c0"] * cfg["c0"] / cfg.get("gamma", 7)
    s.B = B
    s.dt = cfg["dt"]
    s.cell_mult = cfg.get("cell_multiplier", 1.0)
    s.g = _d(cfg.get("gravity", [0, 0, 0]))
    s.lo = _d(cfg["domain_lo"])
    s.hi = _d(cfg["domain_hi"])
    nf = cfg.get("n_fluid", -1)
    s.n_fluid = n if nf is None or nf < 0 else nf
    s.dim = cfg["dim"]
    s.gamma = cfg.get("gamma", 7)
    return s


class SphState:
    """Oracle-side SPH state: columns x, y, z, vx, vy, vz, rho, m (z columns unused in 2D)."""

    def __init__(self, pos, vel, rho, mass, f64=True):
        dt = np.float64 if f64 else np.float32
        self.f64 = f64
        self.n, self.dim = np.asarray(pos).shape
        # always copies: the oracle advances these columns in place
        self.cols = _cols(pos, dt) + _cols(vel, dt) + [np.array(rho, dt, copy=True), np.array(mass, dt, copy=True)]

    def ptrs(self):
        return (ctypes.c_void_p * 8)(*[c.ctypes.data for c in self.cols])

    @property
    def pos(self):
        return np.stack(self.cols[0:self.dim], axis=1)

    @property
    def vel(self):
        return np.stack(self.cols[3:3 + self.dim], axis=1)

    @property
    def rho(self):
        return self.cols[6]


def sph_rates(cfg, state):
    dt = np.float64 if state.f64 else np.float32
    spec = sph_spec(cfg, state.n)
    out = [np.zeros(state.n, dt) for _ in range(4)]
    optr = (ctypes.c_void_p * 4)(*[o.ctypes.data for o in out])
    load().orc_sph_rates(ctypes.byref(spec), 1 if state.f64 else 0, ctypes.c_longlong(state.n), state.ptrs(), optr)
    acc = np.stack(out[:state.dim], axis=1)
    return acc, out[3]


def sph_run(cfg, state, nsteps):
    """Advance the oracle state in place; returns the wall time of the steps in seconds."""
    spec = sph_spec(cfg, state.n)
    return load().orc_sph_run(ctypes.byref(spec), 1 if state.f64 else 0, ctypes.c_longlong(state.n), state.ptrs(),
                              int(nsteps))


_timing = None


def load_timing():
    """The CPU timing build (cpu_timing.cpp: cell-sorted arrays, lists built once per step,
    contraction allowed): the CPU baseline bench.py times."""
    global _timing
    if _timing is None:
        _timing = ctypes.CDLL(_build.build_timing())
        _timing.orc_sph_run_timing.restype = ctypes.c_double
    return _timing


def timing_threads(n=0):
    return load_timing().orc_timing_threads(int(n))


def sph_run_timing(cfg, state, nsteps):
    """Advance the state in place with the CPU timing build; returns the wall time in seconds."""
    spec = sph_spec(cfg, state.n)
    return load_timing().orc_sph_run_timing(ctypes.byref(spec), 1 if state.f64 else 0, ctypes.c_longlong(state.n),
                                            state.ptrs(), int(nsteps))


def sph_stage(cfg, state, stage):
    """Half of an oracle step, in place: 0 = continuity (rho' into rho), 1 = momentum with the
    densities in rho and the update of the fluid's velocities and positions."""
    spec = sph_spec(cfg, state.n)
    rc = load().orc_sph_stage(ctypes.byref(spec), 1 if state.f64 else 0, ctypes.c_longlong(state.n),
                              state.ptrs(), int(stage))
    if rc:
        raise ValueError("stage must be 0 or 1")


def sph_flop_census(cfg, state):
    """Counted flops of one oracle SPH step on `state` (f64, not modified): a dict with the
    particle, candidate and neighbour-pair counts, the flops of the continuity and momentum pair
    loops, of the whole step, and of one candidate test (d and r^2).  Each +, -, *, / and sqrt
    counts one flop."""
    assert state.f64
    spec = sph_spec(cfg, state.n)
    out = np.zeros(7)
    load().orc_sph_flop_census(ctypes.byref(spec), ctypes.c_longlong(state.n), state.ptrs(),
                               out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    keys = ("particles", "candidates", "pairs", "cont_loops", "mom_loops", "step", "test_flops")
    return dict(zip(keys, out.tolist()))


def sph_grad_dual(cfg, state, u, target, nsteps):
    """Forward-mode (dual number) L, dL/dalpha, dL/dB, <dL/dv0, u> with
    L = mean over fluid particles of |x(T) - target|^2."""
    spec = sph_spec(cfg, state.n)
    ucols = _cols(u, np.float64)
    tcols = _cols(target, np.float64)
    uptr = (ctypes.c_void_p * 3)(*[c.ctypes.data for c in ucols])
    tptr = (ctypes.c_void_p * 3)(*[c.ctypes.data for c in tcols])
    out = np.zeros(4)
    load().orc_sph_grad_dual(ctypes.byref(spec), ctypes.c_longlong(state.n), state.ptrs(), uptr, tptr, int(nsteps),
                             _p(out))
    return out


def dem_spec(cfg):
    s = OrcDemSpec()
    s.kn, s.e, s.mu = cfg["kn"], cfg["restitution"], cfg["mu"]
    kt = cfg.get("kt", 0.0)
    s.kt = kt if kt and kt > 0 else cfg["kn"] * 2.0 / 7.0
    s.dt, s.r_max = cfg["dt"], cfg["r_max"]
    s.cell_mult = cfg.get("cell_multiplier", 1.0)
    s.g = _d(cfg.get("gravity", [0, 0, 0]))
    s.lo, s.hi = _d(cfg["domain_lo"]), _d(cfg["domain_hi"])
    s.wall_lo, s.wall_hi = _d(cfg["wall_lo"]), _d(cfg["wall_hi"])
    s.capacity = cfg.get("contact_capacity", 16)
    return s


class DemState:
    def __init__(self, pos, vel, omega, radius, mass, capacity):
        n = np.asarray(pos).shape[0]
        self.n = n
        self.capacity = capacity
        # always copies: the oracle advances these columns in place
        self.cols = (_cols(pos, np.float64) + _cols(vel, np.float64) + _cols(omega, np.float64)
                     + [np.array(radius, np.float64, copy=True), np.array(mass, np.float64, copy=True)])
        self.hpid = np.full(n * capacity, 0xFFFFFFFF, np.uint32)
        self.hxi = np.zeros(n * capacity * 3, np.float64)

    def ptrs(self):
        return (ctypes.c_void_p * 11)(*[c.ctypes.data for c in self.cols])

    @property
    def pos(self):
        return np.stack(self.cols[0:3], axis=1)

    @property
    def vel(self):
        return np.stack(self.cols[3:6], axis=1)

    @property
    def omega(self):
        return np.stack(self.cols[6:9], axis=1)


def dem_run(cfg, state, nsteps):
    """Advance in place; returns (contacts of the last step or -1 on slot overflow, seconds)."""
    spec = dem_spec(cfg)
    sec = ctypes.c_double()
    c = load().orc_dem_run(ctypes.byref(spec), ctypes.c_longlong(state.n), state.ptrs(), _p(state.hpid),
                           _p(state.hxi), int(nsteps), ctypes.byref(sec))
    return c, sec.value
