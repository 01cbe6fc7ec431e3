"""ctypes binding of libprestige_gpu.so (the C ABI declared in include/prestige_gpu.h).

Loading fails loudly when the library is missing: there is no CPU fallback anywhere in the
package.  `build_lib.build()` compiles it (nvcc, sm_103a).
"""
import ctypes
import os

from . import build_lib

PG_OK, PG_EINVAL, PG_ENOMEM, PG_EOVERFLOW, PG_ETIMEOUT, PG_ECUDA, PG_ESTATE, PG_ENOTFOUND = range(8)
PG_F32, PG_F64, PG_U32 = 0, 1, 2
PG_MODEL_SPH, PG_MODEL_DEM = 0, 1
PG_F64_NATIVE, PG_F64_FAST = 0, 1

STATUS_NAMES = {0: "PG_OK", 1: "PG_EINVAL", 2: "PG_ENOMEM", 3: "PG_EOVERFLOW", 4: "PG_ETIMEOUT",
                5: "PG_ECUDA", 6: "PG_ESTATE", 7: "PG_ENOTFOUND"}

_d3 = ctypes.c_double * 3


class PgConfig(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int), ("dim", ctypes.c_int), ("precision", ctypes.c_int), ("gamma", ctypes.c_int),
        ("n_fluid", ctypes.c_longlong),
        ("domain_lo", _d3), ("domain_hi", _d3),
        ("cell_multiplier", ctypes.c_double),
        ("h", ctypes.c_double), ("rho0", ctypes.c_double), ("c0", ctypes.c_double), ("alpha", ctypes.c_double),
        ("eps_av", ctypes.c_double), ("tait_B", ctypes.c_double),
        ("gravity", _d3), ("dt", ctypes.c_double),
        ("kn", ctypes.c_double), ("restitution", ctypes.c_double), ("mu", ctypes.c_double), ("kt", ctypes.c_double),
        ("r_max", ctypes.c_double),
        ("wall_lo", _d3), ("wall_hi", _d3),
        ("contact_capacity", ctypes.c_int),
        ("block_size", ctypes.c_int), ("f64_mode", ctypes.c_int), ("list_capacity", ctypes.c_int),
    ]


class PgInfo(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_longlong),
        ("n_systems", ctypes.c_int), ("dim", ctypes.c_int), ("precision", ctypes.c_int), ("model", ctypes.c_int),
        ("arith", ctypes.c_int),
        ("n_cells", ctypes.c_longlong),
        ("reach", ctypes.c_int), ("pass_grid", ctypes.c_int), ("sort_passes", ctypes.c_int), ("graph", ctypes.c_int),
        ("grid_n", ctypes.c_int * 3), ("grid_lo", _d3), ("cell_size", ctypes.c_double),
        ("list_capacity", ctypes.c_int), ("overlap_split", ctypes.c_longlong),
        ("block_size", ctypes.c_int), ("momentum_block", ctypes.c_int), ("particles_per_warp", ctypes.c_int),
    ]


class PgTiming(ctypes.Structure):
    _fields_ = [("region_ms", ctypes.c_double), ("neighbor_ms", ctypes.c_double), ("gather_ms", ctypes.c_double),
                ("pass_ms", ctypes.c_double), ("steps", ctypes.c_longlong), ("launches", ctypes.c_longlong),
                ("cont_ms", ctypes.c_double), ("list_ms", ctypes.c_double)]


_P = ctypes.c_void_p
_SZ = ctypes.c_size_t
_I = ctypes.c_int
_S = ctypes.c_char_p

# name -> (restype, argtypes).  Every symbol declared in include/prestige_gpu.h.
SIGNATURES = {
    "pg_config_default": (None, [ctypes.POINTER(PgConfig)]),
    "pg_version": (_I, []),
    "pg_create": (_I, [ctypes.POINTER(PgConfig), _SZ, ctypes.POINTER(_P)]),
    "pg_batch_create": (_I, [ctypes.POINTER(PgConfig), ctypes.POINTER(_SZ), _I, ctypes.POINTER(_P)]),
    "pg_destroy": (_I, [_P]),
    "pg_set_field": (_I, [_P, _S, _P, _SZ, _I]),
    "pg_get_field": (_I, [_P, _S, _P, _SZ, _I]),
    "pg_set_field_async": (_I, [_P, _S, _P, _SZ, _I]),
    "pg_get_field_async": (_I, [_P, _S, _P, _SZ, _I]),
    "pg_wait_io": (_I, [_P]),
    "pg_build_neighbors": (_I, [_P]),
    "pg_num_cells": (_I, [_P, ctypes.POINTER(_SZ)]),
    "pg_get_neighbors": (_I, [_P, _P, _P, _P, _SZ]),
    "pg_count_neighbors": (_I, [_P, _P]),
    "pg_get_neighbor_list": (_I, [_P, _P, _P, _SZ, ctypes.POINTER(_SZ)]),
    "pg_get_pair_lists": (_I, [_P, _P, _P, _SZ]),
    "pg_gather_sum": (_I, [_P, _S, _S]),
    "pg_compute_rates": (_I, [_P]),
    "pg_run_equations": (_I, [_P, ctypes.POINTER(_S), _I]),
    "pg_equation_source": (_I, [ctypes.POINTER(_S), _I, _P, _SZ, ctypes.POINTER(_SZ)]),
    "pg_step": (_I, [_P, _I]),
    "pg_step_async": (_I, [_P, _I]),
    "pg_sync": (_I, [_P]),
    "pg_enable_graph": (_I, [_P, _I]),
    "pg_dem_contacts": (_I, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    "pg_dem_get_history": (_I, [_P, _P, _P, _SZ]),
    "pg_dem_set_history": (_I, [_P, _P, _P, _SZ]),
    "pg_forward_checkpointed": (_I, [_P, _I, _I]),
    "pg_backward": (_I, [_P, _P, _P, _P, _P]),
    "pg_autotune": (_I, [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I),
                         ctypes.POINTER(ctypes.c_double)]),
    "pg_set_tuning": (_I, [_P, _I, ctypes.c_double, _I]),
    "pg_set_momentum_block": (_I, [_P, _I]),
    "pg_set_particles_per_warp": (_I, [_P, _I]),
    "pg_step_stage": (_I, [_P, _I]),
    "pg_measure_fma_peaks": (_I, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "pg_timing_enable": (_I, [_P, _I]),
    "pg_timing_read": (_I, [_P, ctypes.POINTER(PgTiming)]),
    "pg_memory_bytes": (_I, [_P, ctypes.POINTER(_SZ)]),
    "pg_get_info": (_I, [_P, ctypes.POINTER(PgInfo)]),
    "pg_cell_list_noalloc": (_I, [_P, _SZ, _I, _P, _P, ctypes.c_double, ctypes.c_double, _P, _P, _P, _SZ,
                                  ctypes.POINTER(_SZ), _P]),
    "pg_last_error": (_S, []),
}

_lib = None


class PgError(RuntimeError):
    def __init__(self, status, func, msg):
        self.status = status
        super().__init__("%s -> %s: %s" % (func, STATUS_NAMES.get(status, status), msg))


def lib_path():
    return build_lib.LIB


def load(build_if_missing=True):
    """Load libprestige_gpu.so (building it first if absent).  Raises if it cannot be had."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("libprestige_gpu.so is not built (%s); run prestige_gb300.build_lib.build()" % path)
        build_lib.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(status, func="pg call"):
    if status != PG_OK:
        msg = load().pg_last_error()
        raise PgError(status, func, msg.decode() if msg else "")
    return status


def default_config():
    c = PgConfig()
    load().pg_config_default(ctypes.byref(c))
    return c


def measure_fma_peaks():
    """(fp64, fp32) FMA-pipe throughput of the current device in TFLOP/s (pg_measure_fma_peaks)."""
    a, b = ctypes.c_double(), ctypes.c_double()
    check(load().pg_measure_fma_peaks(ctypes.byref(a), ctypes.byref(b)), "pg_measure_fma_peaks")
    return a.value, b.value
