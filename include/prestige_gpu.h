/* prestige_gpu.h -- C ABI of the GB300 (sm_103a) particle hot path.
 *
 * The reference (dineshadepu/prestige) describes a pairwise "equation" by the names of the
 * particle slices it reads and writes: the #[equation] macro records them
 * (prestige_macros/src/lib.rs:64-133) into EquationIR.reads / .writes
 * (prestige/src/equations/ir.rs:3-14), fuse() merges equations
 * (prestige/src/equations/fuse.rs:14-40), and the CPU backend runs the fused bodies as a gather
 * into particle i over partners j (prestige/src/codegen/simple_cpu.rs:7-19).  The reference
 * defines no FFI of its own.  This library keeps its contract -- particle data addressed by
 * slice name, i = target, j = partner -- replaces the all-pairs j loop by a cell-list
 * neighbour set, and keeps all state resident on one GPU.  Every entry point below is what a
 * Rust `extern "C"` block (or ctypes) binds in place of the CPU loop; each comment names the
 * reference interface it stands in for.
 *
 * Conventions
 *   - Every call returns a pg_status; pg_last_error() gives a message for the calling thread.
 *   - Host buffers are owned by the caller and only read/written during the call.
 *   - A handle owns its device memory and one CUDA stream.  Calls on one handle must be
 *     serialised by the caller; different handles are independent.
 *   - Per-particle arrays cross the ABI in particle-id order (the order given to
 *     pg_set_field).  Vector fields are interleaved (x0 y0 [z0] x1 y1 ...).
 */
#ifndef PRESTIGE_GPU_H
#define PRESTIGE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PG_VERSION 1

typedef enum pg_status {
  PG_OK = 0,
  PG_EINVAL = 1,    /* bad argument, size or configuration */
  PG_ENOMEM = 2,    /* device allocation failed */
  PG_EOVERFLOW = 3, /* a fixed capacity (contact slots, list capacity) was exceeded */
  PG_ETIMEOUT = 4,  /* a bounded device wait gave up */
  PG_ECUDA = 5,     /* CUDA runtime error (message in pg_last_error) */
  PG_ESTATE = 6,    /* call not valid in the handle's current state */
  PG_ENOTFOUND = 7  /* unknown field name */
} pg_status;

typedef enum pg_dtype { PG_F32 = 0, PG_F64 = 1, PG_U32 = 2 } pg_dtype;

typedef enum pg_model { PG_MODEL_SPH = 0, PG_MODEL_DEM = 1 } pg_model;

/* Pair-kernel arithmetic. */
typedef enum pg_f64_mode {
  PG_F64_NATIVE = 0, /* IEEE arithmetic in the system precision, oracle operation order (bit-exact) */
  PG_F64_FAST = 1    /* f64 systems: double-word arithmetic on the FP32 pipe (f64 tolerance);
                        f32 systems: fused multiply-add allowed */
} pg_f64_mode;

typedef struct pg_config {
  int model;          /* pg_model */
  int dim;            /* 2 or 3 (DEM: 3) */
  int precision;      /* PG_F32 or PG_F64 (DEM: PG_F64) */
  int gamma;          /* Tait exponent (integer, 1..15) */
  long long n_fluid;  /* SPH: ids >= n_fluid (counted from the system's first id) are fixed
                         dummy-wall particles; < 0 means all fluid */
  double domain_lo[3], domain_hi[3]; /* cell-grid extent; particles outside are clamped into edge cells */
  double cell_multiplier;            /* cell side = multiplier * support (1.0 or 0.5) */
  /* SPH */
  double h, rho0, c0, alpha, eps_av, tait_B; /* tait_B <= 0: B = rho0 c0^2 / gamma */
  double gravity[3];
  double dt;
  /* DEM */
  double kn, restitution, mu, kt, r_max;     /* kt <= 0: kt = 2/7 kn */
  double wall_lo[3], wall_hi[3];
  int contact_capacity;
  /* tuning */
  int block_size;     /* threads per block of the SPH list and pair kernels (0: 128; else a multiple of 32, <= 256) */
  int f64_mode;       /* pg_f64_mode */
  int list_capacity;  /* SPH neighbour-list slots per particle (0: 128 in 3D, 64 in 2D); a particle with
                         more neighbours is still handled exactly, by a slower continued walk */
} pg_config;

/* Read-only description of a handle. */
typedef struct pg_info {
  long long n;        /* particles */
  int n_systems, dim, precision, model, arith;
  long long n_cells;  /* all systems */
  int reach;          /* neighbour cells searched on each side */
  int pass_grid;      /* blocks of the persistent pair pass */
  int sort_passes;    /* 8-bit radix passes per step */
  int graph;          /* 1 if steps replay a CUDA graph */
  int grid_n[3];      /* system 0 */
  double grid_lo[3];
  double cell_size;
  int list_capacity;  /* entries per particle of the pair-pass neighbour lists */
  long long overlap_split;  /* > 0: the continuity pass over slots [0, split) runs beside the
                               neighbour lists of [split, n) (double-word SPH handles) */
  int block_size;      /* threads per block of the neighbour lists and the continuity pass */
  int momentum_block;  /* threads per block of the momentum pass */
  int particles_per_warp;  /* target particles per warp of the continuity and momentum passes */
} pg_info;

/* Fill *cfg with defaults (3D f64 SPH, gamma 7, alpha 0.1, eps 0.01, multiplier 1). */
void pg_config_default(pg_config* cfg);
int pg_version(void);

typedef struct pg_system pg_system;

/* Create a system of n particles.  Stands in for the particle slices that a generated
 * `for i in 0..n` loop indexes (prestige/src/codegen/simple_cpu.rs:7; n is unbound there). */
int pg_create(const pg_config* cfg, size_t n, pg_system** out);

/* One handle holding n_systems independent SPH systems, concatenated in id order:
 * system s owns ids [sum_{t<s} counts[t], sum_{t<=s} counts[t]).  All systems share dim,
 * precision, f64_mode and cell_multiplier.  No reference counterpart (the reference runs one
 * loop over one set of slices); it batches many such loops into one launch. */
int pg_batch_create(const pg_config* cfgs, const size_t* counts, int n_systems, pg_system** out);

int pg_destroy(pg_system* sys);

/* Copy a named slice between host and device.  Names are the slice identifiers an equation
 * reads/writes (EquationIR.reads / .writes, prestige/src/equations/ir.rs:8-10):
 *   SPH: "pos" (n*dim), "vel" (n*dim), "rho" (n), "mass" (n); read-only "acc" (n*dim) and
 *        "drho" (n) after pg_compute_rates
 *   DEM: "pos", "vel", "omega" (n*3), "radius" (n), "mass" (n)
 *   any other name: a user scalar slice of n doubles, created by its first pg_set_field
 *        (e.g. "force" of prestige/src/lib.rs:8).
 * dtype PG_F64 or PG_F32 (converted to the stored precision). */
int pg_set_field(pg_system* sys, const char* name, const void* host, size_t count, int dtype);
int pg_get_field(pg_system* sys, const char* name, void* host, size_t count, int dtype);

/* Asynchronous host I/O for step loops that exchange data with the host every step (no
 * reference counterpart: its slices live in host memory).  Host buffers must stay valid, and
 * for inputs unchanged, until pg_wait_io returns; page-locked (pinned) buffers let the copies
 * overlap the steps.  Only fields that exist, in their own precision (dtype = the system's for
 * pos/vel/rho/mass/acc/drho, PG_F64 for user fields).
 *   pg_set_field_async  copies `host` into a staging buffer on an input copy stream; every later
 *                       call on the handle (a step, a rates or neighbour call, a field read)
 *                       first moves it into the field (the buffers trade places; a handle with
 *                       a captured graph copies it in).  So inputs for step k+1 upload while
 *                       step k runs.
 *   pg_get_field_async  snapshots the field at this point of the handle's work (a device copy)
 *                       and copies the snapshot to `host` on an output copy stream; later steps
 *                       do not disturb it.  So results of step k download while step k+1 runs.
 *   pg_wait_io          waits for every copy and step of the handle and reports errors. */
int pg_set_field_async(pg_system* sys, const char* name, const void* host, size_t count, int dtype);
int pg_get_field_async(pg_system* sys, const char* name, void* host, size_t count, int dtype);
int pg_wait_io(pg_system* sys);

/* Neighbour search: cell hash, stable (cell, id) sort, cell-start table.  Replaces the all-pairs
 * `for j in 0..n` of prestige/src/codegen/simple_cpu.rs:8. */
int pg_build_neighbors(pg_system* sys);
int pg_num_cells(pg_system* sys, size_t* n_cells);
/* After pg_build_neighbors: per sorted slot k its cell and particle id; cell_start has
 * n_cells + 1 entries (slots of cell c are cell_start[c] .. cell_start[c+1]). */
int pg_get_neighbors(pg_system* sys, uint32_t* cell_sorted, uint32_t* ids_sorted, uint32_t* cell_start,
                     size_t n_cells_plus_1);
/* Number of neighbours (|x_i - x_j| < support, i itself included) of every particle, id order. */
int pg_count_neighbors(pg_system* sys, uint32_t* counts);
/* CSR neighbour lists in traversal order: offsets (n+1), neighbour ids (capacity entries).
 * *total receives the entry count; PG_EOVERFLOW if it exceeds capacity. */
int pg_get_neighbor_list(pg_system* sys, uint64_t* offsets, uint32_t* neighbors, size_t capacity, size_t* total);
/* The neighbour lists the SPH pair passes read, as the last step or pg_compute_rates built them
 * (sorted-slot order of that neighbour search, pg_get_neighbors): slot k has lengths[k] entries,
 * sorted slots in walk order, at entries[k * list_capacity ...] (min(lengths[k], list_capacity)
 * of them; the passes walk on for the rest).  They are exactly the particles within 2h under
 * the oracle's test in the system's precision (f64 systems: the f64 test, decided in FP32 away
 * from the boundary; f32 systems: the IEEE FP32 test), k itself and coincident particles
 * excluded.  entries may be null (lengths only); capacity counts u32 entries
 * and must be at least n * list_capacity (pg_info.list_capacity). */
int pg_get_pair_lists(pg_system* sys, uint32_t* lengths, uint32_t* entries, size_t capacity);

/* Cell list of n particles that allocates no device memory.  No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc.  Some hosts give all device memory to an
 * allocator of their own (a pool or caching allocator they must not go around).  Others run
 * in loops where cudaMalloc's implicit device synchronisation is not acceptable.
 *
 * Computes the same neighbour search as pg_build_neighbors (cell hash, stable (cell, id) radix
 * sort, cell-start table), bit for bit, for positions already on the device.
 *   pos          device, n * dim doubles, id order (x0 y0 [z0] x1 ...)
 *   grid         domain_lo/hi, support and cell_multiplier as in pg_config
 *   sorted_cell  device, n u32: cell of each sorted slot
 *   sorted_id    device, n u32: particle id of each sorted slot
 *   cell_start   device, cell_start_capacity u32; receives n_cells + 1 entries
 *   n_cells      optional host output: the grid's cell count (also set when the capacity is
 *                too small, so a call with capacity 0 tells the caller how much to pass)
 *   stream       a cudaStream_t, or NULL for the default stream; the call only enqueues work
 * Scratch: a fixed device array compiled into the library, about 8.3 MB, held on every device
 * that uses it until the process exits.  n is limited to 1,048,576 particles; larger n gives
 * PG_EINVAL.  Every call made outside stream capture looks up the array's device address in
 * the current context with cudaGetSymbolAddress (so a cudaDeviceReset or a different context
 * is followed); a call made while `stream` is capturing reuses the address of the last call
 * outside capture on that device, so make one call on each device before capturing
 * (PG_ESTATE otherwise), in the context the capture will use.  Every call shares the array, so
 * calls whose GPU work overlaps (other streams, unordered host threads) race; order them on
 * one stream. */
int pg_cell_list_noalloc(const double* pos, size_t n, int dim, const double domain_lo[3], const double domain_hi[3],
                         double support, double cell_multiplier, uint32_t* sorted_cell, uint32_t* sorted_id,
                         uint32_t* cell_start, size_t cell_start_capacity, size_t* n_cells, void* stream);

/* The body of the reference's eq1 (prestige/src/lib.rs:7-12, `force[i] += mass[j]`) run over
 * the neighbour set instead of all j:  dst[i] += sum_{j : |x_i - x_j| < support} src[j]
 * (j == i included).  dst and src name scalar double slices. */
int pg_gather_sum(pg_system* sys, const char* dst, const char* src);

/* GPU execution of pairwise equations given as source text: the GPU counterpart of the
 * reference's generate_simple_cpu (prestige/src/codegen/simple_cpu.rs:3-22), which only
 * returns the text of `for i in 0..n { for j in 0..n { bodies } }`.  Here the fused bodies run
 * for every particle i and every neighbour j with |x_i - x_j| < support (j == i included), in
 * the traversal order of pg_gather_sum.  Body syntax: `x[i] op= expr` (op: = += -= *= /=) and
 * `let name = expr` statements over slices x[i] / x[j] (user double fields; "mass" and "rho"
 * read-only in double-precision SPH systems), the pair geometry dx dy dz r2 r, `support`, and
 * sqrt exp ln abs min max powi powf sin cos (as calls or Rust methods).  Reads of x[j] see the
 * values before the call.  The kernel is compiled with NVRTC at first use for the device and
 * cached by its source; PG_ESTATE if NVRTC is not available, PG_EINVAL (message in
 * pg_last_error) for a body outside the grammar.  IEEE double without contraction:
 * {"force[i] += mass[j]"} reproduces pg_gather_sum bit for bit. */
int pg_run_equations(pg_system* sys, const char* const* bodies, int n_bodies);
/* The CUDA source pg_run_equations would compile for `bodies` (every slice taken as a double
 * field), for inspection and tests; *needed receives the size including the terminating zero. */
int pg_equation_source(const char* const* bodies, int n_bodies, char* out, size_t capacity, size_t* needed);

/* SPH: evaluate the fused continuity + momentum rates without integrating ("acc" without
 * gravity, "drho").  The GPU form of one generate_simple_cpu loop over the fused SPH equations
 * (prestige/src/equations/fuse.rs:14-40, prestige/src/codegen/simple_cpu.rs:3-22). */
int pg_compute_rates(pg_system* sys);

/* Advance nsteps full steps and wait for them.  SPH step: neighbour search, continuity pass
 * (rho' = rho + dt drho), momentum pass with rho' (v' = v + dt (a + g), x' = x + dt v';
 * wall particles keep x and v).  DEM step: neighbour search, contact pass + integrator.
 * pg_step_async only enqueues them on the handle's stream; pg_sync waits and reports
 * device-side errors (PG_EOVERFLOW for DEM contact slots). */
int pg_step(pg_system* sys, int nsteps);
int pg_step_async(pg_system* sys, int nsteps);
int pg_sync(pg_system* sys);

/* One SPH step in two calls, for hosts that exchange densities between the two passes (a
 * domain split across GPUs, whose halo particles take their densities from the GPU that owns
 * them).  Stage 0: neighbour search, continuity pass, rho' = rho + dt drho into "rho".  Between
 * the stages the caller may replace any densities (pg_set_field or pg_set_field_async of "rho").
 * Stage 1: the packed densities and Tait pressures are refreshed from "rho", then the momentum
 * pass updates v and x.  Stage 0 then stage 1 with nothing in between gives the same bits as
 * pg_step(sys, 1).  PG_ESTATE if stage 1 does not follow a stage 0, or if a step, a neighbour
 * search or a change of another field came in between.  Both calls wait for their work.  No
 * reference counterpart (the reference's loop runs on one set of slices). */
int pg_step_stage(pg_system* sys, int stage);

/* Capture one full step as a CUDA graph; later steps replay it (same results). */
int pg_enable_graph(pg_system* sys, int enable);

/* DEM diagnostics: particle-particle contacts (both sides counted) in the last step. */
int pg_dem_contacts(pg_system* sys, long long* contacts);
/* DEM tangential history, id order: partner ids (n*capacity) and springs (n*capacity*3). */
int pg_dem_get_history(pg_system* sys, uint32_t* partner, double* xi, size_t capacity);
int pg_dem_set_history(pg_system* sys, const uint32_t* partner, const double* xi, size_t capacity);

/* Differentiable SPH (f64, single system).  pg_forward_checkpointed runs nsteps from the current
 * state, keeping the state every `every` steps.  pg_backward then takes dL/dx of the final
 * positions (n*dim, id order) and returns dL/dalpha, dL/dB and dL/dv0 (n*dim, id order); any
 * output pointer may be NULL.  The handle's state stays the final state.  An IEEE handle
 * recomputes each segment from its IEEE checkpoint in the double-word mode (within about 1e-12 of
 * the IEEE trajectory over a segment) and evaluates the adjoint in FP64; its mode, block sizes and
 * graph are restored before the call returns.  No reference counterpart (the reference has no
 * differentiation). */
int pg_forward_checkpointed(pg_system* sys, int nsteps, int every);
int pg_backward(pg_system* sys, const double* dL_dx, double* dL_dalpha, double* dL_dB, double* dL_dv0);

/* Autotuner (SPH handles): time every (cell multiplier 1 or 1/2, arithmetic mode, block size 64,
 * 128 or 256) on the handle's current state for `trial_steps` steps each, keep the fastest whose
 * rates are within the mode's tolerance of the IEEE rates (1e-10 normwise for f64, 1e-4 for
 * f32), then time the momentum pass's own block size (64, 128, 256) with the rest fixed, the
 * common block size again with that momentum block, and, in the tolerance-based modes, the
 * particles per warp of the pair passes (32, 16, 8), apply the result and report it (the
 * momentum block and particles per warp in pg_info).  The handle's state is restored afterwards; a graph-enabled handle
 * is re-captured.  No reference counterpart (the reference has no executable backend to tune). */
int pg_autotune(pg_system* sys, int trial_steps, int* best_block, double* best_multiplier, int* best_f64_mode,
                double* best_ms_per_step);
/* Apply a tuning found earlier (e.g. cached by the host) without searching.  The momentum pass
 * takes the same block size until pg_set_momentum_block sets its own. */
int pg_set_tuning(pg_system* sys, int block, double cell_multiplier, int f64_mode);
/* Block size of the momentum pass alone (64, 128 or 256 threads; 0: the block size of the other
 * list kernels).  pg_autotune chooses it after the other settings: the momentum pass runs alone
 * and reads neighbour records that consecutive slots share, so it can prefer larger blocks than
 * the continuity pass, which shares the SMs with the list kernel. */
int pg_set_momentum_block(pg_system* sys, int block);
/* Target particles per warp of the continuity and momentum passes: 32 (one thread per particle),
 * 16 or 8 (two or four threads share a particle's neighbour list, each summing every second or
 * fourth entry, and their sums are combined in a fixed order).  Only the tolerance-based modes
 * take 16 or 8 (double-word f64, contracted f32: the summation order changes); the IEEE modes
 * keep 32 so that they stay bit-exact.  pg_autotune searches it after the block sizes.  No
 * reference counterpart. */
int pg_set_particles_per_warp(pg_system* sys, int particles_per_warp);

/* Device characterisation: FP64 and FP32 FMA-pipe throughput of the current device in TFLOP/s
 * (two flops per FMA), measured with eight independent FMA chains per thread, 8 blocks of 256
 * threads per SM, timed with CUDA events after a warm-up launch (about 10 ms of GPU time).  These
 * are the denominators of the pair passes' pipe fractions: the IEEE f64 passes run on the FP64
 * pipe, the double-word and f32 passes on the FP32 pipe.  Either pointer may be NULL.  No
 * reference counterpart. */
int pg_measure_fma_peaks(double* fp64_tflops, double* fp32_tflops);

/* Device-side timing of steps (CUDA events on the handle's stream).  The momentum pass time is
 * pass_ms - list_ms - cont_ms.  pg_timing_enable(1) resets
 * the accumulators and makes every later step record events around its stages (steps then run
 * eagerly, not from a graph); pg_timing_read waits for the stream and returns the totals since the
 * last enable. */
typedef struct pg_timing {
  double region_ms;    /* first timed step start -> last timed step end */
  double neighbor_ms;  /* hash + sort + cell table, summed over steps */
  double gather_ms;    /* sorted copies, summed */
  double pass_ms;      /* neighbour lists + pair passes + integrator (DEM: contact pass), summed */
  long long steps;
  long long launches;  /* kernels launched by the timed steps */
  double cont_ms;      /* SPH continuity pass alone (part of pass_ms), summed */
  double list_ms;      /* SPH neighbour-list kernel alone (part of pass_ms), summed */
} pg_timing;
int pg_timing_enable(pg_system* sys, int enable);
int pg_timing_read(pg_system* sys, pg_timing* out);

int pg_memory_bytes(pg_system* sys, size_t* bytes);
int pg_get_info(pg_system* sys, pg_info* info);

/* Message for the last failing call on this thread ("" if none). */
const char* pg_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* PRESTIGE_GPU_H */
