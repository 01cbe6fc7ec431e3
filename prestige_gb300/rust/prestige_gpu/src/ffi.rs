//! Raw bindings of the C ABI in include/prestige_gpu.h: one declaration per entry point, the
//! structs with the header's field order and C layout.  The safe wrapper is in lib.rs.
#![allow(non_camel_case_types, non_snake_case)]

use std::os::raw::{c_char, c_double, c_int, c_longlong, c_void};

pub const PG_VERSION: c_int = 1;

// pg_status
pub const PG_OK: c_int = 0;
pub const PG_EINVAL: c_int = 1;
pub const PG_ENOMEM: c_int = 2;
pub const PG_EOVERFLOW: c_int = 3;
pub const PG_ETIMEOUT: c_int = 4;
pub const PG_ECUDA: c_int = 5;
pub const PG_ESTATE: c_int = 6;
pub const PG_ENOTFOUND: c_int = 7;

// pg_dtype
pub const PG_F32: c_int = 0;
pub const PG_F64: c_int = 1;
pub const PG_U32: c_int = 2;

// pg_model
pub const PG_MODEL_SPH: c_int = 0;
pub const PG_MODEL_DEM: c_int = 1;

// pg_f64_mode
pub const PG_F64_NATIVE: c_int = 0;
pub const PG_F64_FAST: c_int = 1;

/// Opaque handle (`pg_system`).
#[repr(C)]
pub struct pg_system {
    _private: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct pg_config {
    pub model: c_int,
    pub dim: c_int,
    pub precision: c_int,
    pub gamma: c_int,
    pub n_fluid: c_longlong,
    pub domain_lo: [c_double; 3],
    pub domain_hi: [c_double; 3],
    pub cell_multiplier: c_double,
    pub h: c_double,
    pub rho0: c_double,
    pub c0: c_double,
    pub alpha: c_double,
    pub eps_av: c_double,
    pub tait_B: c_double,
    pub gravity: [c_double; 3],
    pub dt: c_double,
    pub kn: c_double,
    pub restitution: c_double,
    pub mu: c_double,
    pub kt: c_double,
    pub r_max: c_double,
    pub wall_lo: [c_double; 3],
    pub wall_hi: [c_double; 3],
    pub contact_capacity: c_int,
    pub block_size: c_int,
    pub f64_mode: c_int,
    pub list_capacity: c_int,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct pg_info {
    pub n: c_longlong,
    pub n_systems: c_int,
    pub dim: c_int,
    pub precision: c_int,
    pub model: c_int,
    pub arith: c_int,
    pub n_cells: c_longlong,
    pub reach: c_int,
    pub pass_grid: c_int,
    pub sort_passes: c_int,
    pub graph: c_int,
    pub grid_n: [c_int; 3],
    pub grid_lo: [c_double; 3],
    pub cell_size: c_double,
    pub list_capacity: c_int,
    pub overlap_split: c_longlong,
    pub block_size: c_int,
    pub momentum_block: c_int,
    pub particles_per_warp: c_int,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct pg_timing {
    pub region_ms: c_double,
    pub neighbor_ms: c_double,
    pub gather_ms: c_double,
    pub pass_ms: c_double,
    pub steps: c_longlong,
    pub launches: c_longlong,
    pub cont_ms: c_double,
    pub list_ms: c_double,
}

extern "C" {
    pub fn pg_config_default(cfg: *mut pg_config);
    pub fn pg_version() -> c_int;

    pub fn pg_create(cfg: *const pg_config, n: usize, out: *mut *mut pg_system) -> c_int;
    pub fn pg_batch_create(cfgs: *const pg_config, counts: *const usize, n_systems: c_int,
                           out: *mut *mut pg_system) -> c_int;
    pub fn pg_destroy(sys: *mut pg_system) -> c_int;

    pub fn pg_set_field(sys: *mut pg_system, name: *const c_char, host: *const c_void, count: usize,
                        dtype: c_int) -> c_int;
    pub fn pg_get_field(sys: *mut pg_system, name: *const c_char, host: *mut c_void, count: usize,
                        dtype: c_int) -> c_int;
    pub fn pg_set_field_async(sys: *mut pg_system, name: *const c_char, host: *const c_void, count: usize,
                              dtype: c_int) -> c_int;
    pub fn pg_get_field_async(sys: *mut pg_system, name: *const c_char, host: *mut c_void, count: usize,
                              dtype: c_int) -> c_int;
    pub fn pg_wait_io(sys: *mut pg_system) -> c_int;

    pub fn pg_build_neighbors(sys: *mut pg_system) -> c_int;
    pub fn pg_num_cells(sys: *mut pg_system, n_cells: *mut usize) -> c_int;
    pub fn pg_get_neighbors(sys: *mut pg_system, cell_sorted: *mut u32, ids_sorted: *mut u32, cell_start: *mut u32,
                            n_cells_plus_1: usize) -> c_int;
    pub fn pg_count_neighbors(sys: *mut pg_system, counts: *mut u32) -> c_int;
    pub fn pg_get_neighbor_list(sys: *mut pg_system, offsets: *mut u64, neighbors: *mut u32, capacity: usize,
                                total: *mut usize) -> c_int;
    pub fn pg_get_pair_lists(sys: *mut pg_system, lengths: *mut u32, entries: *mut u32, capacity: usize) -> c_int;
    pub fn pg_cell_list_noalloc(pos: *const c_double, n: usize, dim: c_int, domain_lo: *const c_double,
                                domain_hi: *const c_double, support: c_double, cell_multiplier: c_double,
                                sorted_cell: *mut u32, sorted_id: *mut u32, cell_start: *mut u32,
                                cell_start_capacity: usize, n_cells: *mut usize, stream: *mut c_void) -> c_int;

    pub fn pg_gather_sum(sys: *mut pg_system, dst: *const c_char, src: *const c_char) -> c_int;
    pub fn pg_run_equations(sys: *mut pg_system, bodies: *const *const c_char, n_bodies: c_int) -> c_int;
    pub fn pg_equation_source(bodies: *const *const c_char, n_bodies: c_int, out: *mut c_char, capacity: usize,
                              needed: *mut usize) -> c_int;

    pub fn pg_compute_rates(sys: *mut pg_system) -> c_int;
    pub fn pg_step(sys: *mut pg_system, nsteps: c_int) -> c_int;
    pub fn pg_step_async(sys: *mut pg_system, nsteps: c_int) -> c_int;
    pub fn pg_step_stage(sys: *mut pg_system, stage: c_int) -> c_int;
    pub fn pg_sync(sys: *mut pg_system) -> c_int;
    pub fn pg_enable_graph(sys: *mut pg_system, enable: c_int) -> c_int;

    pub fn pg_dem_contacts(sys: *mut pg_system, contacts: *mut c_longlong) -> c_int;
    pub fn pg_dem_get_history(sys: *mut pg_system, partner: *mut u32, xi: *mut c_double, capacity: usize) -> c_int;
    pub fn pg_dem_set_history(sys: *mut pg_system, partner: *const u32, xi: *const c_double, capacity: usize)
                              -> c_int;

    pub fn pg_forward_checkpointed(sys: *mut pg_system, nsteps: c_int, every: c_int) -> c_int;
    pub fn pg_backward(sys: *mut pg_system, dL_dx: *const c_double, dL_dalpha: *mut c_double, dL_dB: *mut c_double,
                       dL_dv0: *mut c_double) -> c_int;

    pub fn pg_autotune(sys: *mut pg_system, trial_steps: c_int, best_block: *mut c_int,
                       best_multiplier: *mut c_double, best_f64_mode: *mut c_int, best_ms_per_step: *mut c_double)
                       -> c_int;
    pub fn pg_set_tuning(sys: *mut pg_system, block: c_int, cell_multiplier: c_double, f64_mode: c_int) -> c_int;
    pub fn pg_set_momentum_block(sys: *mut pg_system, block: c_int) -> c_int;
    pub fn pg_set_particles_per_warp(sys: *mut pg_system, particles_per_warp: c_int) -> c_int;
    pub fn pg_measure_fma_peaks(fp64_tflops: *mut c_double, fp32_tflops: *mut c_double) -> c_int;

    pub fn pg_timing_enable(sys: *mut pg_system, enable: c_int) -> c_int;
    pub fn pg_timing_read(sys: *mut pg_system, out: *mut pg_timing) -> c_int;
    pub fn pg_memory_bytes(sys: *mut pg_system, bytes: *mut usize) -> c_int;
    pub fn pg_get_info(sys: *mut pg_system, info: *mut pg_info) -> c_int;

    pub fn pg_last_error() -> *const c_char;
}
