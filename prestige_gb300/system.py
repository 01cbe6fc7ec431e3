"""Host-side handle over the C ABI: named particle slices resident on one GPU.

`ParticleSystem` mirrors how the reference addresses particle data -- by the slice names an
equation reads and writes (prestige_macros/src/lib.rs:64-133, EquationIR.reads/.writes in
prestige/src/equations/ir.rs:3-14) -- and runs the fused pair loop on the GPU instead of the
generated CPU text loop (prestige/src/codegen/simple_cpu.rs:3-22).
"""
import ctypes
import json
import os

import numpy as np

from . import _native as nat

_VEC2 = ("domain_lo", "domain_hi", "gravity", "wall_lo", "wall_hi")


def make_config(**kw):
    """A pg_config from library defaults plus keyword overrides (vectors as 3-sequences)."""
    c = nat.default_config()
    for k, v in kw.items():
        if not hasattr(c, k):
            raise KeyError("unknown config field %r" % k)
        if k in _VEC2:
            arr = getattr(c, k)
            vv = list(v) + [0.0] * (3 - len(v))
            for i in range(3):
                arr[i] = float(vv[i])
        else:
            setattr(c, k, v)
    return c


def config_dict(c):
    out = {}
    for name, _ in nat.PgConfig._fields_:
        v = getattr(c, name)
        out[name] = list(v) if name in _VEC2 else v
    return out


class ParticleSystem:
    """One GPU-resident particle system (or a batch of independent SPH systems)."""

    def __init__(self, config=None, n=0, _handle=None, _counts=None, _configs=None):
        self._lib = nat.load()
        if _handle is not None:
            self._h = _handle
            self.counts = list(_counts)
            self.configs = list(_configs)
        else:
            if config is None:
                config = make_config()
            elif isinstance(config, dict):
                config = make_config(**config)
            h = ctypes.c_void_p()
            nat.check(self._lib.pg_create(ctypes.byref(config), n, ctypes.byref(h)), "pg_create")
            self._h = h
            self.counts = [int(n)]
            self.configs = [config]
        self.config = self.configs[0]
        self.n = int(sum(self.counts))
        self.dim = int(self.config.dim)
        self.f64 = self.config.precision == nat.PG_F64
        self.model = int(self.config.model)

    @classmethod
    def batch(cls, configs, counts):
        lib = nat.load()
        cfgs = [make_config(**c) if isinstance(c, dict) else c for c in configs]
        arr = (nat.PgConfig * len(cfgs))(*cfgs)
        cnt = (ctypes.c_size_t * len(counts))(*[int(x) for x in counts])
        h = ctypes.c_void_p()
        nat.check(lib.pg_batch_create(arr, cnt, len(cfgs), ctypes.byref(h)), "pg_batch_create")
        return cls(_handle=h, _counts=counts, _configs=cfgs)

    # -- lifetime ---------------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.pg_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- fields -------------------------------------------------------------------------------
    def _comps(self, name):
        if name in ("pos", "vel", "acc"):
            return self.dim if self.model == nat.PG_MODEL_SPH else 3
        if name == "omega":
            return 3
        return 1

    def _stored_f64(self, name):
        if self.model == nat.PG_MODEL_SPH and name in ("pos", "vel", "rho", "mass", "acc", "drho"):
            return self.f64
        return True

    def set(self, name, values, dtype=None):
        """Copy a host array into the named slice (id order; vectors interleaved)."""
        if dtype is None:
            dtype = np.float64 if self._stored_f64(name) else np.float32
        a = np.ascontiguousarray(values, dtype=dtype).reshape(-1)
        code = nat.PG_F64 if a.dtype == np.float64 else nat.PG_F32
        nat.check(self._lib.pg_set_field(self._h, name.encode(), a.ctypes.data, a.size, code), "pg_set_field")

    def set_ptr(self, name, ptr, count, f64=True):
        """Copy from a raw host pointer (e.g. pinned memory) into the named slice."""
        nat.check(self._lib.pg_set_field(self._h, name.encode(), ptr, count, nat.PG_F64 if f64 else nat.PG_F32),
                  "pg_set_field")

    def get(self, name, dtype=None):
        if dtype is None:
            dtype = np.float64 if self._stored_f64(name) else np.float32
        comps = self._comps(name)
        out = np.empty(self.n * comps, dtype=dtype)
        code = nat.PG_F64 if out.dtype == np.float64 else nat.PG_F32
        nat.check(self._lib.pg_get_field(self._h, name.encode(), out.ctypes.data, out.size, code), "pg_get_field")
        return out.reshape(self.n, comps) if comps > 1 else out

    def get_ptr(self, name, ptr, count, f64=True):
        nat.check(self._lib.pg_get_field(self._h, name.encode(), ptr, count, nat.PG_F64 if f64 else nat.PG_F32),
                  "pg_get_field")

    def set_ptr_async(self, name, ptr, count, f64=True):
        """Stage a copy from a raw (pinned) host pointer; it takes effect before the next call on
        this handle.  The buffer must stay unchanged until wait_io()."""
        nat.check(self._lib.pg_set_field_async(self._h, name.encode(), ptr, count,
                                               nat.PG_F64 if f64 else nat.PG_F32), "pg_set_field_async")

    def get_ptr_async(self, name, ptr, count, f64=True):
        """Snapshot the named slice now and copy it to a raw (pinned) host pointer in the
        background; the data is there after wait_io()."""
        nat.check(self._lib.pg_get_field_async(self._h, name.encode(), ptr, count,
                                               nat.PG_F64 if f64 else nat.PG_F32), "pg_get_field_async")

    def wait_io(self):
        nat.check(self._lib.pg_wait_io(self._h), "pg_wait_io")

    # -- neighbour search -----------------------------------------------------------------------
    def num_cells(self):
        v = ctypes.c_size_t()
        nat.check(self._lib.pg_num_cells(self._h, ctypes.byref(v)), "pg_num_cells")
        return v.value

    def build_neighbors(self):
        nat.check(self._lib.pg_build_neighbors(self._h), "pg_build_neighbors")

    def neighbors(self):
        """(cell of each sorted slot, id of each sorted slot, cell_start[n_cells + 1])."""
        self.build_neighbors()
        nc = self.num_cells()
        cell = np.empty(self.n, np.uint32)
        ids = np.empty(self.n, np.uint32)
        start = np.empty(nc + 1, np.uint32)
        nat.check(self._lib.pg_get_neighbors(self._h, cell.ctypes.data, ids.ctypes.data, start.ctypes.data, nc + 1),
                  "pg_get_neighbors")
        return cell, ids, start

    def count_neighbors(self):
        out = np.empty(self.n, np.uint32)
        nat.check(self._lib.pg_count_neighbors(self._h, out.ctypes.data), "pg_count_neighbors")
        return out

    def neighbor_list(self):
        offs = np.empty(self.n + 1, np.uint64)
        total = ctypes.c_size_t()
        st = self._lib.pg_get_neighbor_list(self._h, offs.ctypes.data, None, 0, ctypes.byref(total))
        if st not in (nat.PG_OK, nat.PG_EOVERFLOW):
            nat.check(st, "pg_get_neighbor_list")
        nbr = np.empty(max(total.value, 1), np.uint32)
        nat.check(self._lib.pg_get_neighbor_list(self._h, offs.ctypes.data, nbr.ctypes.data, nbr.size,
                                                 ctypes.byref(total)), "pg_get_neighbor_list")
        return offs, nbr[:total.value]

    def pair_lists(self):
        """(lengths, entries) of the pair-pass neighbour lists built by the last step or
        compute_rates: per sorted slot, lengths[k] and entries[k, :min(lengths[k], cap)]
        (sorted slots)."""
        cap = self.info()["list_capacity"]
        lengths = np.empty(self.n, np.uint32)
        entries = np.empty((self.n, cap), np.uint32)
        nat.check(self._lib.pg_get_pair_lists(self._h, lengths.ctypes.data, entries.ctypes.data, entries.size),
                  "pg_get_pair_lists")
        return lengths, entries

    def pair_counts(self):
        """Lengths of the pair-pass neighbour lists built by the last step or compute_rates, per
        sorted slot (exact neighbour counts, the particle itself excluded)."""
        lengths = np.empty(self.n, np.uint32)
        nat.check(self._lib.pg_get_pair_lists(self._h, lengths.ctypes.data, None, 0), "pg_get_pair_lists")
        return lengths

    def run_equations(self, bodies):
        """Run fused pairwise equation bodies (source text) on the GPU over the neighbour set."""
        if isinstance(bodies, str):
            bodies = [bodies]
        arr = (ctypes.c_char_p * len(bodies))(*[b.encode() for b in bodies])
        nat.check(self._lib.pg_run_equations(self._h, arr, len(bodies)), "pg_run_equations")

    def gather_sum(self, dst, src):
        """dst[i] += sum over neighbours j (i included) of src[j]  (eq1 of the reference)."""
        nat.check(self._lib.pg_gather_sum(self._h, dst.encode(), src.encode()), "pg_gather_sum")

    # -- SPH / DEM steps --------------------------------------------------------------------------
    def compute_rates(self):
        nat.check(self._lib.pg_compute_rates(self._h), "pg_compute_rates")
        return self.get("acc"), self.get("drho")

    def step(self, nsteps=1):
        nat.check(self._lib.pg_step(self._h, int(nsteps)), "pg_step")

    def step_stage(self, stage):
        """Half a step: 0 = neighbour search and continuity pass (rho' into "rho"), 1 = the
        momentum pass with the densities in "rho" (which the caller may replace in between)."""
        nat.check(self._lib.pg_step_stage(self._h, int(stage)), "pg_step_stage")

    def step_async(self, nsteps=1):
        nat.check(self._lib.pg_step_async(self._h, int(nsteps)), "pg_step_async")

    def sync(self):
        nat.check(self._lib.pg_sync(self._h), "pg_sync")

    def enable_graph(self, enable=True):
        nat.check(self._lib.pg_enable_graph(self._h, 1 if enable else 0), "pg_enable_graph")

    def dem_contacts(self):
        v = ctypes.c_longlong()
        nat.check(self._lib.pg_dem_contacts(self._h, ctypes.byref(v)), "pg_dem_contacts")
        return v.value

    def dem_history(self):
        C = self.config.contact_capacity
        pid = np.empty(self.n * C, np.uint32)
        xi = np.empty(self.n * C * 3, np.float64)
        nat.check(self._lib.pg_dem_get_history(self._h, pid.ctypes.data, xi.ctypes.data, C), "pg_dem_get_history")
        return pid.reshape(self.n, C), xi.reshape(self.n, C, 3)

    def set_dem_history(self, pid, xi):
        C = self.config.contact_capacity
        pid = np.ascontiguousarray(pid, np.uint32).reshape(-1)
        xi = np.ascontiguousarray(xi, np.float64).reshape(-1)
        nat.check(self._lib.pg_dem_set_history(self._h, pid.ctypes.data, xi.ctypes.data, C), "pg_dem_set_history")

    # -- differentiation ----------------------------------------------------------------------------
    def forward_checkpointed(self, nsteps, every):
        nat.check(self._lib.pg_forward_checkpointed(self._h, int(nsteps), int(every)), "pg_forward_checkpointed")

    def backward(self, dL_dx):
        g = np.ascontiguousarray(dL_dx, np.float64).reshape(-1)
        da = ctypes.c_double()
        dB = ctypes.c_double()
        dv0 = np.empty(self.n * self.dim, np.float64)
        nat.check(self._lib.pg_backward(self._h, g.ctypes.data, ctypes.addressof(da), ctypes.addressof(dB),
                                        dv0.ctypes.data), "pg_backward")
        return da.value, dB.value, dv0.reshape(self.n, self.dim)

    # -- tuning and introspection ---------------------------------------------------------------------
    def tuning_key(self):
        """Cache key of a tuning: dimension, precision and particle-count bucket (powers of 2)."""
        bucket = 1 << max(self.n - 1, 0).bit_length()
        return "dim%d-%s-n%d" % (self.dim, "f64" if self.f64 else "f32", bucket)

    def autotune(self, trial_steps=3, cache=None):
        """Run pg_autotune, or apply the cached result for this handle's key when `cache` (a JSON
        file path) holds one.  A new result is written to the cache."""
        key = self.tuning_key()
        if cache is not None and os.path.exists(cache):
            with open(cache) as f:
                table = json.load(f)
            if key in table:
                t = table[key]
                self.set_tuning(t["block_size"], t["cell_multiplier"], t["f64_mode"])
                self.set_momentum_block(t.get("momentum_block", 0))
                self.set_particles_per_warp(t.get("particles_per_warp", 32))
                return dict(t, cached=True)
        blk = ctypes.c_int()
        mult = ctypes.c_double()
        mode = ctypes.c_int()
        ms = ctypes.c_double()
        nat.check(self._lib.pg_autotune(self._h, int(trial_steps), ctypes.byref(blk), ctypes.byref(mult),
                                        ctypes.byref(mode), ctypes.byref(ms)), "pg_autotune")
        res = {"block_size": blk.value, "cell_multiplier": mult.value, "f64_mode": mode.value,
               "momentum_block": self.info()["momentum_block"],
               "particles_per_warp": self.info()["particles_per_warp"], "ms_per_step": ms.value}
        if cache is not None:
            table = {}
            if os.path.exists(cache):
                with open(cache) as f:
                    table = json.load(f)
            table[key] = res
            tmp = cache + ".tmp"
            with open(tmp, "w") as f:
                json.dump(table, f, indent=1, sort_keys=True)
            os.replace(tmp, cache)
        return dict(res, cached=False)

    def set_tuning(self, block_size, cell_multiplier, f64_mode):
        nat.check(self._lib.pg_set_tuning(self._h, int(block_size), float(cell_multiplier), int(f64_mode)),
                  "pg_set_tuning")

    def set_particles_per_warp(self, ppw):
        """Target particles per warp of the continuity and momentum passes (32, 16 or 8; the IEEE
        modes always run 32)."""
        nat.check(self._lib.pg_set_particles_per_warp(self._h, int(ppw)), "pg_set_particles_per_warp")

    def set_momentum_block(self, block_size):
        """Block size of the momentum pass alone (0: the other list kernels' block size)."""
        nat.check(self._lib.pg_set_momentum_block(self._h, int(block_size)), "pg_set_momentum_block")

    def info(self):
        i = nat.PgInfo()
        nat.check(self._lib.pg_get_info(self._h, ctypes.byref(i)), "pg_get_info")
        return {name: (list(getattr(i, name)) if name in ("grid_n", "grid_lo") else getattr(i, name))
                for name, _ in nat.PgInfo._fields_}

    def timing_enable(self, enable=True):
        nat.check(self._lib.pg_timing_enable(self._h, 1 if enable else 0), "pg_timing_enable")

    def timing_read(self):
        t = nat.PgTiming()
        nat.check(self._lib.pg_timing_read(self._h, ctypes.byref(t)), "pg_timing_read")
        return {name: getattr(t, name) for name, _ in nat.PgTiming._fields_}

    def memory_bytes(self):
        v = ctypes.c_size_t()
        nat.check(self._lib.pg_memory_bytes(self._h, ctypes.byref(v)), "pg_memory_bytes")
        return v.value
