"""The cell list that allocates no device memory (pg_cell_list_noalloc).

Some callers cannot call cudaMalloc: hosts whose device memory all belongs to an allocator of
their own, and loops where cudaMalloc's implicit synchronisation is not acceptable.  For them
the library offers a cell list whose scratch is a fixed array compiled into the library.  These
tests call it through the C ABI with device buffers the test owns. Two calls in a row must each
give the same sorted cells, sorted ids and cell table as the handle-based neighbour search
(pg_build_neighbors / pg_get_neighbors), bit for bit. The second call follows the first without
any reset of the shared scratch.

This file is named to be collected last: the shared scratch must not depend on what ran before.
"""
import ctypes

import numpy as np
import pytest

from prestige_gb300 import ParticleSystem, _native, make_config, workloads

MAX_PARTICLES = 1 << 20


def _reference_cell_list(w):
    cfg = w["config"]
    s = ParticleSystem(make_config(**cfg), w["n"])
    s.set("pos", w["fields"]["pos"])
    cell, ids, start = s.neighbors()
    s.close()
    return cell, ids, start


def _noalloc_cell_list(w):
    import torch

    lib = _native.load()
    cfg = w["config"]
    n, dim = w["n"], cfg["dim"]
    pos = torch.tensor(np.ascontiguousarray(w["fields"]["pos"], np.float64).reshape(-1), device="cuda")
    lo = (ctypes.c_double * 3)(*cfg["domain_lo"])
    hi = (ctypes.c_double * 3)(*cfg["domain_hi"])
    support = 2.0 * cfg["h"]
    mult = cfg.get("cell_multiplier", 1.0)
    ncells = ctypes.c_size_t(0)
    # capacity 0: the call only reports the cell count
    st = lib.pg_cell_list_noalloc(pos.data_ptr(), n, dim, lo, hi, support, mult, None, None, None, 0,
                                  ctypes.byref(ncells), None)
    assert st == _native.PG_EINVAL and ncells.value > 0
    cell = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    ids = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    start = torch.full((ncells.value + 1,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    st = lib.pg_cell_list_noalloc(pos.data_ptr(), n, dim, lo, hi, support, mult, cell.data_ptr(), ids.data_ptr(),
                                  start.data_ptr(), start.numel(), ctypes.byref(ncells), None)
    assert st == _native.PG_OK, lib.pg_last_error()
    torch.cuda.synchronize()
    as_u32 = lambda t: t.cpu().numpy().view(np.uint32)
    return as_u32(cell), as_u32(ids), as_u32(start)


@pytest.mark.gpu
def test_noalloc_cell_list_matches_handle_path_twice_in_a_row(pg):
    cases = [workloads.sph_lattice_3d(n=50000, seed=12),
             workloads.dam_break_2d(dx=0.03)]
    for w in cases:  # two calls in a row, different grids and sizes, shared scratch not reset
        got = _noalloc_cell_list(w)
        ref = _reference_cell_list(w)
        for g, r in zip(got, ref):
            assert np.array_equal(g, r)


@pytest.mark.gpu
def test_noalloc_cell_list_at_its_size_limit(pg):
    """Exactly the largest accepted size: the scratch's key, value and histogram areas are full."""
    w = workloads.sph_lattice_3d(n=MAX_PARTICLES, seed=14, cell_multiplier=0.5)
    got = _noalloc_cell_list(w)
    ref = _reference_cell_list(w)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)


@pytest.mark.gpu
def test_noalloc_cell_list_of_no_particles(pg):
    """n = 0 with null position and sort buffers: only the cell table is written, all zeros."""
    import torch

    lib = _native.load()
    w = workloads.sph_lattice_3d(n=1000, seed=2)
    cfg = w["config"]
    lo = (ctypes.c_double * 3)(*cfg["domain_lo"])
    hi = (ctypes.c_double * 3)(*cfg["domain_hi"])
    ncells = ctypes.c_size_t(0)
    st = lib.pg_cell_list_noalloc(None, 0, 3, lo, hi, 2.0 * cfg["h"], 1.0, None, None, None, 0,
                                  ctypes.byref(ncells), None)
    assert st == _native.PG_EINVAL and ncells.value > 0
    start = torch.full((ncells.value + 1,), -1, dtype=torch.int32, device="cuda")
    st = lib.pg_cell_list_noalloc(None, 0, 3, lo, hi, 2.0 * cfg["h"], 1.0, None, None, start.data_ptr(),
                                  start.numel(), ctypes.byref(ncells), None)
    assert st == _native.PG_OK, lib.pg_last_error()
    torch.cuda.synchronize()
    assert (start.cpu().numpy() == 0).all()


def test_noalloc_rejects_sizes_beyond_its_limit(pg):
    lib = _native.load()
    lo = (ctypes.c_double * 3)(0.0, 0.0, 0.0)
    hi = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
    ncells = ctypes.c_size_t(0)
    st = lib.pg_cell_list_noalloc(None, MAX_PARTICLES + 1, 3, lo, hi, 0.1, 1.0, None, None, None, 0,
                                  ctypes.byref(ncells), None)
    assert st == _native.PG_EINVAL
    assert b"limit" in lib.pg_last_error()
