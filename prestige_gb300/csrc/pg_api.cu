// C ABI of the library (declared in include/prestige_gpu.h).
//
// The reference addresses particle data by the names of the slices an equation reads and
// writes (prestige_macros/src/lib.rs:64-133 -> EquationIR.reads / .writes,
// prestige/src/equations/ir.rs:3-14) and runs a fused set of equations as one gather loop
// (prestige/src/equations/fuse.rs:14-40, prestige/src/codegen/simple_cpu.rs:3-22).  A handle
// here owns those named slices on the GPU and runs the fused neighbour-search + pair + integrate
// step on one CUDA stream; host buffers are only touched inside a call.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <chrono>
#include <cmath>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "pg_arith.cuh"
#include "pg_internal.cuh"
#include "pg_kernels.cuh"
#include "pg_system.cuh"

using namespace pg;

namespace pg {

namespace {

constexpr double kPi = 3.14159265358979323846;

int arith_of(const pg_config& c, int f64) {
  if (f64) return c.f64_mode == PG_F64_FAST ? ARITH_F64_DF : ARITH_F64_EXACT;
  return c.f64_mode == PG_F64_FAST ? ARITH_F32_FAST : ARITH_F32_EXACT;
}

// SPH constants of one system, both precisions, with the formulas of the oracle's
// sph_kernel_factors / sph_consts (this file is compiled with -ffp-contract=off).
SphK make_sphk(const pg_config& c, const Grid& g, uint32_t cell_base, uint32_t id_begin, uint32_t id_end,
               uint32_t fluid_end) {
  SphK k;
  memset(&k, 0, sizeof(k));
  k.g = grid_k(g, cell_base);
  const double h = c.h;
  const double sigma = c.dim == 2 ? 10.0 / (7.0 * kPi * h * h) : 1.0 / (kPi * h * h * h);
  const double fa = sigma / (h * h);
  const double fb = -0.75 * sigma / h;
  const double B = c.tait_B > 0.0 ? c.tait_B : c.rho0 * c.c0 * c.c0 / (double)c.gamma;
  k.d.fa = fa;
  k.d.fb = fb;
  k.d.inv_h = 1.0 / h;
  k.d.four_h2 = (2.0 * h) * (2.0 * h);
  k.d.avk = (-2.0 * c.c0 * h) * c.alpha;
  k.avk_alpha = -2.0 * c.c0 * h;
  k.d.eps_h2 = c.eps_av * h * h;
  k.d.B = B;
  k.d.inv_rho0 = 1.0 / c.rho0;
  k.d.dt = c.dt;
  for (int d = 0; d < 3; ++d) k.d.g[d] = c.gravity[d];
  k.f.fa = (float)fa;
  k.f.fb = (float)fb;
  k.f.inv_h = (float)(1.0 / h);
  k.f.four_h2 = (float)((2.0 * h) * (2.0 * h));
  k.f.avk = (float)(-2.0 * c.c0 * h) * (float)c.alpha;
  k.f.eps_h2 = (float)(c.eps_av * h * h);
  k.f.B = (float)B;
  k.f.inv_rho0 = (float)(1.0 / c.rho0);
  k.f.dt = (float)c.dt;
  for (int d = 0; d < 3; ++d) k.f.g[d] = (float)c.gravity[d];
  df_split(k.d.fa, &k.w.fa[0], &k.w.fa[1]);
  df_split(k.d.fb, &k.w.fb[0], &k.w.fb[1]);
  df_split(k.d.inv_h, &k.w.inv_h[0], &k.w.inv_h[1]);
  df_split(k.d.four_h2, &k.w.four_h2[0], &k.w.four_h2[1]);
  df_split(k.d.avk, &k.w.avk[0], &k.w.avk[1]);
  df_split(k.d.eps_h2, &k.w.eps_h2[0], &k.w.eps_h2[1]);
  df_split(k.d.B, &k.w.B[0], &k.w.B[1]);
  df_split(k.d.inv_rho0, &k.w.inv_rho0[0], &k.w.inv_rho0[1]);
  df_split(-3.0 * fa, &k.w.near0[0], &k.w.near0[1]);
  df_split(2.25 * fa / h, &k.w.near1[0], &k.w.near1[1]);
  df_split(-4.0 * fb / h, &k.w.far0[0], &k.w.far0[1]);
  df_split(fb / (h * h), &k.w.far1[0], &k.w.far1[1]);
  df_split(4.0 * fb, &k.w.far2[0], &k.w.far2[1]);
  k.w.h2 = (float)(h * h);
  k.w.band = (float)(1e-9 * k.d.four_h2);
  k.two_h_f = (float)(2.0 * h) * 1.0000001f;
  k.pos_pad = 8.0 * h;
  k.id_begin = id_begin;
  k.id_end = id_end;
  k.fluid_end = fluid_end;
  k.gamma = c.gamma;
  return k;
}

int validate_sph(const pg_config& c) {
  if (c.dim != 2 && c.dim != 3) {
    set_error("dim must be 2 or 3 (got %d)", c.dim);
    return PG_EINVAL;
  }
  if (c.precision != PG_F32 && c.precision != PG_F64) {
    set_error("precision must be PG_F32 or PG_F64");
    return PG_EINVAL;
  }
  if (!(c.h > 0) || !(c.rho0 > 0) || !(c.c0 > 0) || !(c.dt >= 0) || !(c.alpha >= 0) || !(c.eps_av > 0)) {
    set_error("SPH parameters must satisfy h > 0, rho0 > 0, c0 > 0, dt >= 0, alpha >= 0, eps > 0");
    return PG_EINVAL;
  }
  if (c.gamma < 1 || c.gamma > 15) {
    set_error("gamma must be an integer in 1..15 (got %d)", c.gamma);
    return PG_EINVAL;
  }
  if (c.f64_mode != PG_F64_NATIVE && c.f64_mode != PG_F64_FAST) {
    set_error("f64_mode must be PG_F64_NATIVE or PG_F64_FAST");
    return PG_EINVAL;
  }
  return PG_OK;
}

int validate_dem(const pg_config& c) {
  if (c.dim != 3 || c.precision != PG_F64) {
    set_error("DEM systems are 3D and double precision");
    return PG_EINVAL;
  }
  if (!(c.kn > 0) || !(c.restitution > 0 && c.restitution <= 1) || !(c.mu >= 0) || !(c.r_max > 0) || !(c.dt >= 0)) {
    set_error("DEM parameters must satisfy kn > 0, 0 < e <= 1, mu >= 0, r_max > 0, dt >= 0");
    return PG_EINVAL;
  }
  if (c.contact_capacity < 1 || c.contact_capacity > 256) {
    set_error("contact_capacity must be in 1..256");
    return PG_EINVAL;
  }
  return PG_OK;
}

}  // namespace

size_t pg_elem_bytes(const pg_system* s) { return s->f64 ? 8 : 4; }

// Allocate the sorted packed arrays for the current arithmetic mode.
int ensure_sorted_buffers(pg_system* s) {
  size_t sz[6];
  sph_sorted_layout(s->arith, sz);
  const size_t n = s->n ? s->n : 1;
  for (int i = 0; i < 6; ++i)
    if (sz[i]) PG_TRY(s->sorted[i].ensure(sz[i] * (n + kPackPad)));
  PG_TRY(s->nlist.ensure(4 * ((n + kListTile - 1) / kListTile) * kListTile * (size_t)s->list_cap));
  // per list entry: {m_j F, u} (double-word, 16 B, written by the continuity pass and read by the
  // momentum pass of the same step) or the pair values of the IEEE step (pg_sph_sym.cu)
  const size_t entries = ((n + kListTile - 1) / kListTile) * kListTile * (size_t)s->list_cap;
  if (s->arith == ARITH_F64_DF) PG_TRY(s->fcache.ensure(16 * entries));
  if (s->arith == ARITH_F64_EXACT) PG_TRY(s->fcache.ensure(sph_sym_entry_bytes() * entries));
  PG_TRY(s->nlen.ensure(4 * n));
  PG_TRY(s->nresume.ensure(8 * n));
  PG_TRY(s->posmin.ensure(3 * sizeof(unsigned long long) * (size_t)s->nsys));
  return PG_OK;
}

SphArgs sph_args(pg_system* s, int integrate, bool rates) {
  SphArgs a;
  memset(&a, 0, sizeof(a));
  a.sys = s->sphk.as<SphK>();
  a.sys_of_id = s->nsys > 1 ? s->sys_of_id.as<uint32_t>() : nullptr;
  a.n = (uint32_t)s->n;
  a.dim = s->dim;
  a.reach = s->grids[0].reach;
  a.sorted_cell = s->nw.sorted_cell;
  a.sorted_id = s->nw.sorted_id;
  a.cell_start = s->nw.cell_start.as<uint32_t>();
  for (int i = 0; i < 6; ++i) a.s[i] = s->sorted[i].p;
  a.s[6] = a.s[7] = nullptr;
  a.pos = s->pos.p;
  a.vel = s->vel.p;
  a.rho = s->rho.p;
  a.mass = s->mass.p;
  a.acc = rates ? s->acc.p : nullptr;
  a.drho = rates ? s->drho.p : nullptr;
  a.integrate = integrate;
  a.nlist = s->nlist.as<uint32_t>();
  a.nlen = s->nlen.as<uint32_t>();
  a.nresume = s->nresume.as<uint32_t>();
  a.fcache = s->arith == ARITH_F64_DF || s->arith == ARITH_F64_EXACT ? s->fcache.p : nullptr;
  a.cap = (uint32_t)s->list_cap;
  a.err = s->err.as<unsigned>();
  a.posmin = s->posmin.as<unsigned long long>();
  a.k_begin = 0;
  a.k_end = (uint32_t)s->n;
  return a;
}

NbrArgs nbr_args(pg_system* s) {
  NbrArgs a;
  memset(&a, 0, sizeof(a));
  a.grid = s->gridk.as<GridK>();
  a.sys_of_id = s->nsys > 1 ? s->sys_of_id.as<uint32_t>() : nullptr;
  a.n = (uint32_t)s->n;
  a.dim = s->dim;
  a.reach = s->grids[0].reach;
  a.f64 = s->f64;
  a.sorted_cell = s->nw.sorted_cell;
  a.sorted_id = s->nw.sorted_id;
  a.cell_start = s->nw.cell_start.as<uint32_t>();
  a.spos = s->spos.p;
  return a;
}

// Hash + stable sort + cell table for the current positions (enqueued on the stream).
int enqueue_neighbors(pg_system* s) {
  s->stage_pending = false;  // any neighbour search ends a pending pg_step_stage(0)
  const void* pos = s->pos.p;
  // the double-word packs need each system's minimum position of the step (sph_gather_df)
  unsigned long long* posmin = nullptr;
  if (s->model == PG_MODEL_SPH && s->arith == ARITH_F64_DF && s->posmin.p) {
    posmin = s->posmin.as<unsigned long long>();
    PG_CUDA_TRY(cudaMemsetAsync(posmin, 0xff, 3 * sizeof(unsigned long long) * (size_t)s->nsys, s->stream));
  }
  PG_TRY(launch_hash(s->stream, s->gridk.as<GridK>(), s->nsys > 1 ? s->sys_of_id.as<uint32_t>() : nullptr, s->f64,
                     s->dim, pos, s->n, s->nw.keys[0].as<uint32_t>(), s->nw.vals[0].as<uint32_t>(), posmin));
  PG_TRY(sort_and_table(s->stream, s->nw));
  return PG_OK;
}

int mom_block(const pg_system* s) { return s->block_mom > 0 ? s->block_mom : s->block; }

// Kernels enqueued by one neighbour search (hash, radix passes, cell-start table).
long long neighbor_launches(const pg_system* s) { return 1 + 3LL * s->nw.passes + 1; }

// The continuity part of a step: neighbour search, sorted gather, neighbour lists and the
// continuity pass (rho' into the canonical density and the sorted pack).  ev (optional): events
// 0-4 of a step (start, after the neighbour search, after the sorted gather, after the lists,
// after the continuity pass).
// The IEEE f64 step evaluates each pair once (pg_sph_sym.cu: four kernels) from 16,384 particles;
// below, where the step is bound by the latency of its launches, the two-sided passes (two
// kernels) are faster: the 6,518-particle dam break took 0.149 against 0.125 ms per step.  Both
// give the oracle's bits.
constexpr size_t kPairOnceMin = 16384;
bool pair_once(const pg_system* s) { return s->arith == ARITH_F64_EXACT && s->n >= kPairOnceMin; }

int enqueue_sph_front(pg_system* s, cudaEvent_t* ev) {
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[0], s->stream));
  PG_TRY(enqueue_neighbors(s));
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[1], s->stream));
  SphArgs a = sph_args(s, 1, false);
  PG_TRY(launch_sph_gather(s->stream, a, s->arith));
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[2], s->stream));
  if (s->arith == ARITH_F64_EXACT && s->ov_split > 0 && s->ov_split < s->n) {
    // each pair once (pg_sph_sym.cu); the lists of [split, n) on the auxiliary stream beside the
    // lists of [0, split), then the pair values of the slots whose partners all lie below split,
    // the rest once every list is built
    SphArgs a1 = a, a2 = a;
    a1.k_end = s->ov_split;
    a2.k_begin = s->ov_split;
    PG_CUDA_TRY(cudaEventRecord(s->ov_ev[0], s->stream));
    PG_CUDA_TRY(cudaStreamWaitEvent(s->aux, s->ov_ev[0], 0));
    PG_TRY(launch_sph_list(s->aux, a2, s->arith, s->ov_list_grid, s->block));
    PG_CUDA_TRY(cudaEventRecord(s->ov_ev[1], s->aux));
    PG_TRY(launch_sph_list(s->stream, a1, s->arith, s->list_grid, s->block));
    s->list_arith = s->arith;
    if (ev) PG_CUDA_TRY(cudaEventRecord(ev[3], s->stream));
    PG_TRY(launch_sph_sym(s->stream, a1, 0, s->block, s->ov_split, 0));
    PG_CUDA_TRY(cudaStreamWaitEvent(s->stream, s->ov_ev[1], 0));
    PG_TRY(launch_sph_sym(s->stream, a, 0, s->block, s->ov_split, 1));
    PG_TRY(launch_sph_sym(s->stream, a, 1, s->block));
    if (ev) PG_CUDA_TRY(cudaEventRecord(ev[4], s->stream));
    s->launches += neighbor_launches(s) + 6;
    return PG_OK;
  }
  if (pair_once(s)) {
    // each pair once (pg_sph_sym.cu): the pair values of a slot need its partners' complete lists
    PG_TRY(launch_sph_list(s->stream, a, s->arith, s->list_grid, s->block));
    s->list_arith = s->arith;
    if (ev) PG_CUDA_TRY(cudaEventRecord(ev[3], s->stream));
    PG_TRY(launch_sph_sym(s->stream, a, 0, s->block));
    PG_TRY(launch_sph_sym(s->stream, a, 1, s->block));
    if (ev) PG_CUDA_TRY(cudaEventRecord(ev[4], s->stream));
    s->launches += neighbor_launches(s) + 4;
    return PG_OK;
  }
  if (s->ov_split > 0 && s->ov_split < s->n) {
    // lists of [0, split) first; then the continuity pass over them runs beside the lists of
    // [split, n) on the auxiliary stream, which goes on with the continuity pass over
    // [split, n) (neither continuity launch reads the packed rho' the other writes); the
    // momentum pass needs every rho', so it runs last
    SphArgs a1 = a, a2 = a;
    a1.k_end = s->ov_split;
    a2.k_begin = s->ov_split;
    PG_TRY(launch_sph_list(s->stream, a1, s->arith, s->list_grid, s->block));
    s->list_arith = s->arith;
    if (ev) PG_CUDA_TRY(cudaEventRecord(ev[3], s->stream));
    PG_CUDA_TRY(cudaEventRecord(s->ov_ev[0], s->stream));
    PG_CUDA_TRY(cudaStreamWaitEvent(s->aux, s->ov_ev[0], 0));
    PG_TRY(launch_sph_list(s->aux, a2, s->arith, s->ov_list_grid, s->block));
    PG_TRY(launch_sph_list_pass(s->aux, a2, s->arith, SPH_CONT, 0, s->block, s->lanes));  // one block per tile
    PG_CUDA_TRY(cudaEventRecord(s->ov_ev[1], s->aux));
    PG_TRY(launch_sph_list_pass(s->stream, a1, s->arith, SPH_CONT, s->ov_pass_grid, s->block, s->lanes));
    PG_CUDA_TRY(cudaStreamWaitEvent(s->stream, s->ov_ev[1], 0));
    if (ev) PG_CUDA_TRY(cudaEventRecord(ev[4], s->stream));
    s->launches += neighbor_launches(s) + 5;
    return PG_OK;
  }
  PG_TRY(launch_sph_list(s->stream, a, s->arith, s->list_grid, s->block));
  s->list_arith = s->arith;
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[3], s->stream));
  PG_TRY(launch_sph_list_pass(s->stream, a, s->arith, SPH_CONT, s->pass_grid[SPH_CONT], s->block, s->lanes));
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[4], s->stream));
  s->launches += neighbor_launches(s) + 3;
  return PG_OK;
}

// The momentum part of a step: the momentum pass with the packed rho' (velocity and position
// update).  ev (optional): event 5 of a step (end).
int enqueue_sph_momentum(pg_system* s, cudaEvent_t* ev) {
  SphArgs a = sph_args(s, 1, false);
  if (pair_once(s)) {
    PG_TRY(launch_sph_sym(s->stream, a, 2, mom_block(s)));
    PG_TRY(launch_sph_sym(s->stream, a, 3, mom_block(s)));
    s->launches += 2;
    if (ev) PG_CUDA_TRY(cudaEventRecord(ev[5], s->stream));
    return PG_OK;
  }
  PG_TRY(launch_sph_list_pass(s->stream, a, s->arith, SPH_MOM, s->pass_grid[SPH_MOM], mom_block(s), s->lanes));
  s->launches += 1;
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[5], s->stream));
  return PG_OK;
}

// ev (optional): 6 events recorded at stage boundaries (start, after the neighbour search,
// after the sorted gather, after the neighbour lists, after the continuity pass, end).
int enqueue_sph_step(pg_system* s, bool rates, int integrate, cudaEvent_t* ev) {
  if (!rates) {
    PG_TRY(enqueue_sph_front(s, ev));
    return enqueue_sph_momentum(s, ev);
  }
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[0], s->stream));
  PG_TRY(enqueue_neighbors(s));
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[1], s->stream));
  SphArgs a = sph_args(s, integrate, rates);
  PG_TRY(launch_sph_gather(s->stream, a, s->arith));
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[2], s->stream));
  PG_TRY(launch_sph_list(s->stream, a, s->arith, s->list_grid, s->block));
  s->list_arith = s->arith;
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[3], s->stream));
  PG_TRY(launch_sph_list_pass(s->stream, a, s->arith, SPH_RATES, s->pass_grid[SPH_RATES], s->block));
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[4], s->stream));
  s->launches += neighbor_launches(s) + 3;
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[5], s->stream));
  return PG_OK;
}

DemArgs dem_args(pg_system* s) {
  DemArgs a;
  memset(&a, 0, sizeof(a));
  a.K = s->demk.as<DemK>();
  a.n = (uint32_t)s->n;
  a.reach = s->grids[0].reach;
  a.sorted_cell = s->nw.sorted_cell;
  a.sorted_id = s->nw.sorted_id;
  a.cell_start = s->nw.cell_start.as<uint32_t>();
  a.sA = s->sorted[0].as<double4_32a>();
  a.sB = s->sorted[1].as<double4_32a>();
  a.sW = s->sorted[2].as<double4_32a>();
  a.sF = s->sorted[3].as<float4>();
  a.pos = s->pos.as<double>();
  a.vel = s->vel.as<double>();
  a.omega = s->omega.as<double>();
  a.radius = s->radius.as<double>();
  a.mass = s->mass.as<double>();
  a.hpid_old = s->hpid[s->hcur].as<uint32_t>();
  a.hxi_old = s->hxi[s->hcur].as<double>();
  a.hpid_new = s->hpid[s->hcur ^ 1].as<uint32_t>();
  a.hxi_new = s->hxi[s->hcur ^ 1].as<double>();
  a.contacts = s->contacts.as<unsigned long long>();
  a.err = s->err.as<unsigned>();
  return a;
}

int enqueue_dem_step(pg_system* s, cudaEvent_t* ev) {
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[0], s->stream));
  PG_TRY(enqueue_neighbors(s));
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[1], s->stream));
  DemArgs a = dem_args(s);
  PG_TRY(launch_dem_gather(s->stream, a));
  PG_CUDA_TRY(cudaMemsetAsync(s->contacts.p, 0, sizeof(unsigned long long), s->stream));
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[2], s->stream));
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[3], s->stream));
  PG_TRY(launch_dem_pass(s->stream, a));
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[4], s->stream));
  if (ev) PG_CUDA_TRY(cudaEventRecord(ev[5], s->stream));
  s->launches += neighbor_launches(s) + 2;
  return PG_OK;
}

constexpr int kStepEvents = 6;

// Events for one timed step, from the handle's event pool (created once, reused every step).
int timing_events(pg_system* s, cudaEvent_t** out) {
  while (s->ev_pool.size() < kStepEvents) {
    cudaEvent_t e;
    PG_CUDA_TRY(cudaEventCreate(&e));
    s->ev_pool.push_back(e);
  }
  for (int i = 0; i < kStepEvents; ++i) {
    s->ev_pending.push_back(s->ev_pool.back());
    s->ev_pool.pop_back();
  }
  *out = &s->ev_pending[s->ev_pending.size() - kStepEvents];
  return PG_OK;
}

// Fold the pending step events into the accumulators (stream must be idle).
int timing_collect(pg_system* s) {
  for (size_t b = 0; b + kStepEvents <= s->ev_pending.size(); b += kStepEvents) {
    cudaEvent_t* e = &s->ev_pending[b];
    float t01, t12, t23, t34, t25;
    PG_CUDA_TRY(cudaEventElapsedTime(&t01, e[0], e[1]));
    PG_CUDA_TRY(cudaEventElapsedTime(&t12, e[1], e[2]));
    PG_CUDA_TRY(cudaEventElapsedTime(&t23, e[2], e[3]));
    PG_CUDA_TRY(cudaEventElapsedTime(&t34, e[3], e[4]));
    PG_CUDA_TRY(cudaEventElapsedTime(&t25, e[2], e[5]));
    s->tacc.neighbor_ms += t01;
    s->tacc.gather_ms += t12;
    s->tacc.pass_ms += t25;
    s->tacc.list_ms += t23;
    s->tacc.cont_ms += t34;
    s->tacc.steps += 1;
  }
  // region: first start -> last end of the pending batch, added to the running region total
  if (s->ev_pending.size() >= kStepEvents) {
    float reg;
    PG_CUDA_TRY(cudaEventElapsedTime(&reg, s->ev_pending.front(), s->ev_pending.back()));
    s->tacc.region_ms += reg;
  }
  for (cudaEvent_t e : s->ev_pending) s->ev_pool.push_back(e);
  s->ev_pending.clear();
  return PG_OK;
}

// One full step, enqueued; flips the DEM history buffers.
int enqueue_step(pg_system* s) {
  cudaEvent_t* ev = nullptr;
  if (s->timing) PG_TRY(timing_events(s, &ev));
  if (s->model == PG_MODEL_DEM) {
    if (!ev && s->graph_enabled && s->graph_exec[s->hcur]) {
      PG_CUDA_TRY(cudaGraphLaunch(s->graph_exec[s->hcur], s->stream));
      s->launches += neighbor_launches(s) + 2;
    } else {
      PG_TRY(enqueue_dem_step(s, ev));
    }
    s->hcur ^= 1;
    return PG_OK;
  }
  if (!ev && s->graph_enabled && s->graph_exec[0]) {
    PG_CUDA_TRY(cudaGraphLaunch(s->graph_exec[0], s->stream));
    s->launches += neighbor_launches(s) + 4;
    return PG_OK;
  }
  return enqueue_sph_step(s, false, 1, ev);
}

// Wait for the stream and report device-side errors.
int sync_and_check(pg_system* s) {
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  unsigned e = 0;
  PG_CUDA_TRY(cudaMemcpy(&e, s->err.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
  if (e) {
    PG_CUDA_TRY(cudaMemset(s->err.p, 0, sizeof(unsigned)));
    if (e & ERR_CONTACT_OVERFLOW) {
      set_error("a particle had more than contact_capacity (%d) contacts; history of the extra contacts was dropped",
                s->cfg.contact_capacity);
      return PG_EOVERFLOW;
    }
    set_error("device error word 0x%x", e);
    return PG_ECUDA;
  }
  return PG_OK;
}

void drop_graphs(pg_system* s) {
  for (int i = 0; i < 2; ++i)
    if (s->graph_exec[i]) {
      cudaGraphExecDestroy(s->graph_exec[i]);
      s->graph_exec[i] = nullptr;
    }
}

int capture_graphs(pg_system* s) {
  drop_graphs(s);
  const int ngraphs = s->model == PG_MODEL_DEM ? 2 : 1;
  const int hsave = s->hcur;
  for (int gi = 0; gi < ngraphs; ++gi) {
    s->hcur = gi;
    cudaGraph_t graph = nullptr;
    PG_CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    const long long l0 = s->launches;
    int st = s->model == PG_MODEL_DEM ? enqueue_dem_step(s, nullptr) : enqueue_sph_step(s, false, 1, nullptr);
    s->launches = l0;
    cudaError_t ce = cudaStreamEndCapture(s->stream, &graph);
    if (st != PG_OK) {
      if (graph) cudaGraphDestroy(graph);
      s->hcur = hsave;
      return st;
    }
    if (ce != cudaSuccess) {
      s->hcur = hsave;
      set_error("graph capture failed: %s", cudaGetErrorString(ce));
      return PG_ECUDA;
    }
    // node priorities: the overlapped step's list kernel keeps its stream's priority in a graph
    cudaError_t ie = cudaGraphInstantiate(&s->graph_exec[gi], graph, cudaGraphInstantiateFlagUseNodePriority);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
      s->hcur = hsave;
      set_error("graph instantiation failed: %s", cudaGetErrorString(ie));
      return PG_ECUDA;
    }
  }
  s->hcur = hsave;
  return PG_OK;
}

// Overlap of the continuity pass (FMA-bound) with the list kernel (ALU-bound) for double-word
// SPH handles of at least 1M particles: the lists of the first 70 % of the slots are built
// first, then the continuity pass over them runs beside the lists of the rest, and the
// continuity pass over the rest follows those lists on their stream.  The list kernel's
// persistent grid leaves room on every SM for two thirds of the pass's blocks (registers per
// block from the kernels' attributes) and runs on a stream of the highest priority, so its
// blocks are placed first; the continuity passes run one block per tile and fill the SMs as the
// list blocks finish.  Measured at 4M particles (ms per step):
//   no overlap, persistent grids                                          9.46
//   overlap with both kernels on persistent grids                        9.27
//   the same build later: persistent grids 8.10, backfilling pass 8.11,
//   backfilling pass and list-stream priority 7.76
//   continuity over the rest on the list stream                           7.65 (7.70 without)
//   splits 0.5 / 0.6 / 0.8 of the slots                                   7.92 / 7.72 / 7.69
//   the same after the per-entry cache held u (7.02 at 0.7): 0.6 / 0.8    7.02 / 7.05
// A finer pipeline (the slots in 4, 8 or 16 even chunks, each chunk's continuity pass starting
// when its lists are done) gave 7.80 / 7.84 / 8.02 ms against 7.76 for two chunks on the same
// box: lists and continuity add up to about 4.4 ms however they are interleaved, so once the SMs
// are backfilled the two kernels share a saturated machine.
// At 1M particles it is even (1.965 ms either way), at 256k slower (0.690 against 0.670 ms),
// hence the threshold.  The 512-system batch of 2D dam breaks (6.1M particles, one handle)
// gains too: 3.36 against 3.45 ms (with persistent grids it had lost, 3.91 against 3.81).
// The auxiliary stream of the overlapped schedules (greatest priority: the list kernel's blocks
// are placed first, the pair pass beside it fills the rest) and its two events.
int ensure_aux_stream(pg_system* s) {
  if (!s->aux) {
    int least = 0, greatest = 0;
    PG_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    PG_CUDA_TRY(cudaStreamCreateWithPriority(&s->aux, cudaStreamNonBlocking, greatest));
  }
  for (int i = 0; i < 2; ++i)
    if (!s->ov_ev[i]) PG_CUDA_TRY(cudaEventCreateWithFlags(&s->ov_ev[i], cudaEventDisableTiming));
  return PG_OK;
}

int choose_overlap(pg_system* s, int sms) {
  s->ov_split = 0;
  if (s->model == PG_MODEL_SPH && s->arith == ARITH_F64_EXACT && s->n >= 1000000) {
    // IEEE step: the lists of the last three quarters of the slots (ALU work) beside the pair
    // values (FP64 work) of the slots of the first quarter whose partners all lie in it
    const int locc = sph_list_occupancy(s->arith, s->dim, -1, s->block);
    if (locc < 1) return PG_OK;
    PG_TRY(ensure_aux_stream(s));
    s->ov_pass_grid = 0;
    s->ov_list_grid = std::max(1, locc / 2) * sms;
    s->ov_split = (uint32_t)(s->n / 4 / (size_t)s->block * (size_t)s->block);
    return PG_OK;
  }
  if (s->model != PG_MODEL_SPH || s->arith != ARITH_F64_DF || s->n < 1000000) return PG_OK;
  const int rp = sph_list_regs(s->arith, s->dim, SPH_CONT, s->lanes), rl = sph_list_regs(s->arith, s->dim, -1);
  if (rp <= 0 || rl <= 0) return PG_OK;
  const int per_block_p = ((rp + 7) / 8) * 8 * s->block, per_block_l = ((rl + 7) / 8) * 8 * s->block;
  const int regs = 65536, threads = 2048;
  int bp = std::max(1, (regs / per_block_p) * 2 / 3);
  int bl = (regs - bp * per_block_p) / per_block_l;
  bl = std::min(bl, (threads - bp * s->block) / s->block);
  if (bl < 1) return PG_OK;
  PG_TRY(ensure_aux_stream(s));
  // the continuity pass beside the lists runs one block per tile, so the block scheduler fills
  // the SMs with it as the list kernel's blocks finish
  s->ov_pass_grid = 0;
  s->ov_list_grid = bl * sms;
  s->ov_split = (uint32_t)(s->n * 7 / 10 / (size_t)s->block * (size_t)s->block);
  return PG_OK;
}

int choose_pass_grid(pg_system* s) {
  int dev = 0, sms = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev));
  PG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  for (int st = 0; st < 3; ++st) {
    const int occ = sph_list_occupancy(s->arith, s->dim, st, st == SPH_MOM ? mom_block(s) : s->block, s->lanes);
    s->pass_grid[st] = occ > 0 ? occ * sms : 0;  // persistent: one resident wave
  }
  const int locc = sph_list_occupancy(s->arith, s->dim, -1, s->block);
  s->list_grid = locc > 0 ? locc * sms : 0;
  return choose_overlap(s, sms);
}

// Cell grids of every system, their device copies and the neighbour-search workspace.
int build_grids(pg_system* s, std::vector<GridK>& gk) {
  const int ns = s->nsys;
  s->grids.resize(ns);
  gk.resize(ns);
  uint64_t cell_base = 0;
  for (int i = 0; i < ns; ++i) {
    const pg_config& c = s->cfgs[i];
    const double support = s->model == PG_MODEL_DEM ? 2.0 * c.r_max : 2.0 * c.h;
    PG_TRY(make_grid(c.dim, c.domain_lo, c.domain_hi, support, c.cell_multiplier, &s->grids[i]));
    gk[i] = grid_k(s->grids[i], (uint32_t)cell_base);
    cell_base += s->grids[i].ncells();
    if (cell_base >= 0xFFFFFFF0ull) {
      set_error("batch: total cell count exceeds the 32-bit cell index");
      return PG_EINVAL;
    }
  }
  for (int i = 1; i < ns; ++i)
    if (s->grids[i].reach != s->grids[0].reach) {
      set_error("batch: all systems must use the same cell multiplier");
      return PG_EINVAL;
    }
  s->ncells = cell_base;
  PG_TRY(s->gridk.ensure(sizeof(GridK) * ns));
  PG_CUDA_TRY(cudaMemcpy(s->gridk.p, gk.data(), sizeof(GridK) * ns, cudaMemcpyHostToDevice));
  PG_TRY(s->nw.init(s->n, s->ncells));
  return PG_OK;
}

// SPH per-system constants (device table).
int build_sph_tables(pg_system* s, const std::vector<GridK>& gk) {
  const int ns = s->nsys;
  std::vector<SphK> k(ns);
  for (int i = 0; i < ns; ++i) {
    const pg_config& c = s->cfgs[i];
    const size_t cnt = s->id_begin[i + 1] - s->id_begin[i];
    const size_t nf = c.n_fluid < 0 || (size_t)c.n_fluid > cnt ? cnt : (size_t)c.n_fluid;
    k[i] = make_sphk(c, s->grids[i], gk[i].cell_base, (uint32_t)s->id_begin[i], (uint32_t)s->id_begin[i + 1],
                     (uint32_t)(s->id_begin[i] + nf));
  }
  PG_TRY(s->sphk.ensure(sizeof(SphK) * ns));
  PG_CUDA_TRY(cudaMemcpy(s->sphk.p, k.data(), sizeof(SphK) * ns, cudaMemcpyHostToDevice));
  return PG_OK;
}

// Build grids, tables and buffers for the handle's configuration(s).
int setup_system(pg_system* s) {
  const int ns = s->nsys;
  std::vector<GridK> gk;
  PG_TRY(build_grids(s, gk));
  if (ns > 1) {
    std::vector<uint32_t> soi(s->n);
    for (int i = 0; i < ns; ++i)
      for (size_t k = s->id_begin[i]; k < s->id_begin[i + 1]; ++k) soi[k] = (uint32_t)i;
    PG_TRY(s->sys_of_id.ensure(4 * (s->n ? s->n : 1)));
    if (s->n) PG_CUDA_TRY(cudaMemcpy(s->sys_of_id.p, soi.data(), 4 * s->n, cudaMemcpyHostToDevice));
  }
  const size_t n = s->n ? s->n : 1;
  PG_TRY(s->err.ensure(sizeof(unsigned)));
  PG_CUDA_TRY(cudaMemset(s->err.p, 0, sizeof(unsigned)));
  if (s->model == PG_MODEL_SPH) {
    PG_TRY(build_sph_tables(s, gk));
    const size_t eb = pg_elem_bytes(s);
    PG_TRY(s->pos.ensure(eb * n * s->dim));
    PG_TRY(s->vel.ensure(eb * n * s->dim));
    PG_TRY(s->rho.ensure(eb * n));
    PG_TRY(s->mass.ensure(eb * n));
    PG_CUDA_TRY(cudaMemset(s->pos.p, 0, eb * n * s->dim));
    PG_CUDA_TRY(cudaMemset(s->vel.p, 0, eb * n * s->dim));
    PG_CUDA_TRY(cudaMemset(s->rho.p, 0, eb * n));
    PG_CUDA_TRY(cudaMemset(s->mass.p, 0, eb * n));
    PG_TRY(ensure_sorted_buffers(s));
    PG_TRY(choose_pass_grid(s));
  } else {
    const pg_config& c = s->cfgs[0];
    DemK k;
    memset(&k, 0, sizeof(k));
    k.g = gk[0];
    k.kn = c.kn;
    k.kt = c.kt > 0 ? c.kt : c.kn * 2.0 / 7.0;
    k.mu = c.mu;
    k.dt = c.dt;
    const double le = std::log(c.restitution);
    k.gcoef = -2.0 * le / std::sqrt(kPi * kPi + le * le);
    for (int d = 0; d < 3; ++d) {
      k.grav[d] = c.gravity[d];
      k.wall_lo[d] = c.wall_lo[d];
      k.wall_hi[d] = c.wall_hi[d];
      k.wall_lo_f[d] = (float)c.wall_lo[d];
      k.wall_hi_f[d] = (float)c.wall_hi[d];
    }
    k.capacity = c.contact_capacity;
    k.dt_finite = std::isfinite(c.dt) ? 1 : 0;
    PG_TRY(s->demk.ensure(sizeof(DemK)));
    PG_CUDA_TRY(cudaMemcpy(s->demk.p, &k, sizeof(DemK), cudaMemcpyHostToDevice));
    PG_TRY(s->pos.ensure(8 * n * 3));
    PG_TRY(s->vel.ensure(8 * n * 3));
    PG_TRY(s->omega.ensure(8 * n * 3));
    PG_TRY(s->radius.ensure(8 * n));
    PG_TRY(s->mass.ensure(8 * n));
    PG_CUDA_TRY(cudaMemset(s->pos.p, 0, 8 * n * 3));
    PG_CUDA_TRY(cudaMemset(s->vel.p, 0, 8 * n * 3));
    PG_CUDA_TRY(cudaMemset(s->omega.p, 0, 8 * n * 3));
    PG_CUDA_TRY(cudaMemset(s->radius.p, 0, 8 * n));
    PG_CUDA_TRY(cudaMemset(s->mass.p, 0, 8 * n));
    for (int i = 0; i < 3; ++i) PG_TRY(s->sorted[i].ensure(32 * n));
    PG_TRY(s->sorted[3].ensure(16 * n));
    const size_t C = (size_t)c.contact_capacity;
    for (int b = 0; b < 2; ++b) {
      PG_TRY(s->hpid[b].ensure(4 * n * C));
      PG_TRY(s->hxi[b].ensure(8 * n * C * 3));
      PG_CUDA_TRY(cudaMemset(s->hpid[b].p, 0xFF, 4 * n * C));
      PG_CUDA_TRY(cudaMemset(s->hxi[b].p, 0, 8 * n * C * 3));
    }
    PG_TRY(s->contacts.ensure(sizeof(unsigned long long)));
    PG_CUDA_TRY(cudaMemset(s->contacts.p, 0, sizeof(unsigned long long)));
  }
  return PG_OK;
}

// Re-derive grids, tables, sorted-pack layout and launch shapes of an SPH handle for a new cell
// multiplier, arithmetic mode and block size.  The particle state is kept; graphs are dropped
// (re-captured by the caller if it wants them).
int retune_sph(pg_system* s, double mult, int f64_mode, int block) {
  if (s->model != PG_MODEL_SPH) {
    set_error("tuning applies to SPH handles");
    return PG_EINVAL;
  }
  if (!(mult > 0.0) || (f64_mode != PG_F64_NATIVE && f64_mode != PG_F64_FAST) || block < 32 ||
      block > kSphMaxThreads || block % 32) {
    set_error("invalid tuning (multiplier %g, f64_mode %d, block %d)", mult, f64_mode, block);
    return PG_EINVAL;
  }
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  drop_graphs(s);
  for (auto& c : s->cfgs) {
    c.cell_multiplier = mult;
    c.f64_mode = f64_mode;
    c.block_size = block;
  }
  s->cfg = s->cfgs[0];
  std::vector<GridK> gk;
  PG_TRY(build_grids(s, gk));
  PG_TRY(build_sph_tables(s, gk));
  s->arith = arith_of(s->cfg, s->f64);
  s->block = block;
  s->block_mom = 0;
  s->lanes = 1;
  PG_TRY(ensure_sorted_buffers(s));
  PG_TRY(choose_pass_grid(s));
  s->nbr_valid = false;
  return PG_OK;
}

int set_momentum_block(pg_system* s, int block) {
  if (s->model != PG_MODEL_SPH) {
    set_error("tuning applies to SPH handles");
    return PG_EINVAL;
  }
  if (block != 0 && (block < 32 || block > kSphMaxThreads || block % 32)) {
    set_error("momentum block %d must be 0 or a multiple of 32 in 32..%d", block, kSphMaxThreads);
    return PG_EINVAL;
  }
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  drop_graphs(s);
  s->block_mom = block;
  return choose_pass_grid(s);
}

int set_pass_lanes(pg_system* s, int lanes) {
  if (s->model != PG_MODEL_SPH) {
    set_error("tuning applies to SPH handles");
    return PG_EINVAL;
  }
  if (lanes != 1 && lanes != 2 && lanes != 4) {
    set_error("lanes per particle %d must be 1, 2 or 4 (32, 16 or 8 particles per warp)", lanes);
    return PG_EINVAL;
  }
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  drop_graphs(s);
  s->lanes = lanes;
  return choose_pass_grid(s);
}

// Field lookup: returns the buffer, its element count per particle and whether it is stored
// in the system precision (else double).
DevBuf* find_field(pg_system* s, const char* name, int* comps, bool* sys_prec, bool* writable) {
  *writable = true;
  *sys_prec = false;
  *comps = 1;
  const std::string nm(name);
  if (s->model == PG_MODEL_SPH) {
    *sys_prec = true;
    if (nm == "pos") { *comps = s->dim; return &s->pos; }
    if (nm == "vel") { *comps = s->dim; return &s->vel; }
    if (nm == "rho") return &s->rho;
    if (nm == "mass") return &s->mass;
    if (nm == "acc") { *comps = s->dim; *writable = false; return s->acc.p ? &s->acc : nullptr; }
    if (nm == "drho") { *writable = false; return s->drho.p ? &s->drho : nullptr; }
    *sys_prec = false;
  } else {
    if (nm == "pos") { *comps = 3; return &s->pos; }
    if (nm == "vel") { *comps = 3; return &s->vel; }
    if (nm == "omega") { *comps = 3; return &s->omega; }
    if (nm == "radius") return &s->radius;
    if (nm == "mass") return &s->mass;
  }
  auto it = s->user.find(nm);
  if (it != s->user.end()) return it->second.get();
  return nullptr;
}

int io_streams(pg_system* s) {
  if (!s->io_in) PG_CUDA_TRY(cudaStreamCreateWithFlags(&s->io_in, cudaStreamNonBlocking));
  if (!s->io_out) PG_CUDA_TRY(cudaStreamCreateWithFlags(&s->io_out, cudaStreamNonBlocking));
  return PG_OK;
}

int io_slot(pg_system* s, const std::string& name, pg_system::IoSlot** out) {
  PG_TRY(io_streams(s));
  pg_system::IoSlot& sl = s->io[name];
  if (!sl.in_ready) {
    for (cudaEvent_t* e : {&sl.in_ready, &sl.in_free, &sl.snap_ready, &sl.snap_free})
      PG_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    PG_CUDA_TRY(cudaEventRecord(sl.in_free, s->stream));
    PG_CUDA_TRY(cudaEventRecord(sl.snap_free, s->io_out));
  }
  *out = &sl;
  return PG_OK;
}

// Moves the inputs staged by pg_set_field_async into their fields, on the compute stream, before
// any later work of the handle.
int apply_io_inputs(pg_system* s) {
  for (auto& kv : s->io) {
    pg_system::IoSlot& sl = kv.second;
    if (!sl.pending) continue;
    int comps;
    bool sys_prec, writable;
    DevBuf* b = find_field(s, kv.first.c_str(), &comps, &sys_prec, &writable);
    sl.pending = false;
    if (!b) continue;
    PG_CUDA_TRY(cudaStreamWaitEvent(s->stream, sl.in_ready, 0));
    if (!s->graph_enabled && sl.in_bytes && sl.in_bytes == b->bytes && sl.stage.bytes == b->bytes) {
      // the staging buffer becomes the field and the field the next staging buffer: kernels take
      // the field pointers when they are enqueued, so no copy is needed (a captured graph holds
      // the old pointers, hence the copy below for graph handles); the work enqueued before this
      // point still reads the old field, and the next upload into it waits for in_free
      std::swap(b->p, sl.stage.p);
    } else if (sl.in_bytes) {
      PG_CUDA_TRY(cudaMemcpyAsync(b->p, sl.stage.p, sl.in_bytes, cudaMemcpyDeviceToDevice, s->stream));
    }
    PG_CUDA_TRY(cudaEventRecord(sl.in_free, s->stream));
    s->nbr_valid = false;
  }
  return PG_OK;
}

}  // namespace pg

pg_system::~pg_system() {
  if (aux) cudaStreamSynchronize(aux);
  for (cudaEvent_t e : ov_ev)
    if (e) cudaEventDestroy(e);
  if (aux) cudaStreamDestroy(aux);
  if (io_in) cudaStreamSynchronize(io_in);
  if (io_out) cudaStreamSynchronize(io_out);
  for (auto& kv : io)
    for (cudaEvent_t e : {kv.second.in_ready, kv.second.in_free, kv.second.snap_ready, kv.second.snap_free})
      if (e) cudaEventDestroy(e);
  if (io_in) cudaStreamDestroy(io_in);
  if (io_out) cudaStreamDestroy(io_out);
  drop_graphs(this);
  for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
  for (cudaEvent_t e : ev_pending) cudaEventDestroy(e);
  destroy_adjoint(this);
  if (stream) cudaStreamDestroy(stream);
}

// =========================================================================================
// extern "C"
// =========================================================================================
extern "C" {

const char* pg_last_error(void) { return pg::last_error(); }

int pg_version(void) { return PG_VERSION; }

void pg_config_default(pg_config* c) {
  if (!c) return;
  memset(c, 0, sizeof(*c));
  c->model = PG_MODEL_SPH;
  c->dim = 3;
  c->precision = PG_F64;
  c->gamma = 7;
  c->n_fluid = -1;
  for (int d = 0; d < 3; ++d) {
    c->domain_lo[d] = 0.0;
    c->domain_hi[d] = 1.0;
    c->wall_lo[d] = 0.0;
    c->wall_hi[d] = 1.0;
  }
  c->cell_multiplier = 1.0;
  c->h = 0.013;
  c->rho0 = 1000.0;
  c->c0 = 10.0;
  c->alpha = 0.1;
  c->eps_av = 0.01;
  c->tait_B = 0.0;
  c->dt = 1e-4;
  c->kn = 1e5;
  c->restitution = 0.9;
  c->mu = 0.3;
  c->kt = 0.0;
  c->r_max = 1e-3;
  c->contact_capacity = 16;
  c->block_size = 0;
  c->f64_mode = PG_F64_NATIVE;
  c->list_capacity = 0;
}

static int create_common(const pg_config* cfgs, const size_t* counts, int nsys, pg_system** out) {
  pg::clear_error();
  if (!cfgs || !counts || !out || nsys < 1) {
    pg::set_error("null argument or n_systems < 1");
    return PG_EINVAL;
  }
  *out = nullptr;
  const pg_config& c0 = cfgs[0];
  if (c0.model != PG_MODEL_SPH && c0.model != PG_MODEL_DEM) {
    pg::set_error("unknown model %d", c0.model);
    return PG_EINVAL;
  }
  if (c0.model == PG_MODEL_DEM && nsys != 1) {
    pg::set_error("batched handles hold SPH systems only");
    return PG_EINVAL;
  }
  size_t total = 0;
  for (int i = 0; i < nsys; ++i) {
    const pg_config& c = cfgs[i];
    int st = c0.model == PG_MODEL_SPH ? validate_sph(c) : validate_dem(c);
    if (st != PG_OK) return st;
    if (c.model != c0.model || c.dim != c0.dim || c.precision != c0.precision || c.f64_mode != c0.f64_mode ||
        c.cell_multiplier != c0.cell_multiplier) {
      pg::set_error("batch: systems must share model, dim, precision, f64_mode and cell_multiplier");
      return PG_EINVAL;
    }
    total += counts[i];
  }
  if (total >= 0xFFFFFFF0ull) {
    pg::set_error("too many particles (%zu); ids are 32-bit", total);
    return PG_EINVAL;
  }
  std::unique_ptr<pg_system> s(new pg_system());
  s->cfg = c0;
  s->cfgs.assign(cfgs, cfgs + nsys);
  s->model = c0.model;
  s->dim = c0.dim;
  s->f64 = c0.precision == PG_F64;
  s->arith = arith_of(c0, s->f64);
  if (c0.list_capacity < 0 || c0.list_capacity > 4096) {
    pg::set_error("list_capacity must be in 0..4096 (got %d)", c0.list_capacity);
    return PG_EINVAL;
  }
  s->list_cap = c0.list_capacity > 0 ? c0.list_capacity : (c0.dim == 2 ? 64 : 128);
  if (c0.block_size != 0 && (c0.block_size < 32 || c0.block_size > kSphMaxThreads || c0.block_size % 32)) {
    pg::set_error("block_size must be 0 or a multiple of 32 in 32..%d (got %d)", kSphMaxThreads, c0.block_size);
    return PG_EINVAL;
  }
  s->block = c0.block_size > 0 ? c0.block_size : kSphThreads;
  s->n = total;
  s->nsys = nsys;
  s->id_begin.assign(nsys + 1, 0);
  for (int i = 0; i < nsys; ++i) s->id_begin[i + 1] = s->id_begin[i] + counts[i];
  PG_CUDA_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  int st = pg::setup_system(s.get());
  if (st != PG_OK) return st;
  PG_CUDA_TRY(cudaDeviceSynchronize());
  *out = s.release();
  return PG_OK;
}

int pg_create(const pg_config* cfg, size_t n, pg_system** out) { return create_common(cfg, &n, 1, out); }

int pg_batch_create(const pg_config* cfgs, const size_t* counts, int n_systems, pg_system** out) {
  return create_common(cfgs, counts, n_systems, out);
}

int pg_destroy(pg_system* s) {
  if (!s) return PG_OK;
  cudaStreamSynchronize(s->stream);
  delete s;
  return PG_OK;
}

// Every entry point starts here: inputs staged by pg_set_field_async take effect before the call.
static int check(pg_system* s) {
  pg::clear_error();
  if (!s) {
    pg::set_error("null handle");
    return PG_EINVAL;
  }
  return s->io.empty() ? PG_OK : pg::apply_io_inputs(s);
}

// Field, element count and byte size for the asynchronous copies (system precision only).
static int io_field(pg_system* s, const char* name, const void* host, size_t count, int dtype, bool input,
                    pg::DevBuf** out, size_t* bytes) {
  if (!name || (!host && count)) {
    pg::set_error("null name or buffer");
    return PG_EINVAL;
  }
  int comps;
  bool sys_prec, writable;
  pg::DevBuf* b = pg::find_field(s, name, &comps, &sys_prec, &writable);
  if (!b) {
    pg::set_error("unknown field '%s' (asynchronous copies need an existing field)", name);
    return PG_ENOTFOUND;
  }
  if (input && !writable) {
    pg::set_error("field '%s' is read-only", name);
    return PG_EINVAL;
  }
  if (count != s->n * (size_t)comps) {
    pg::set_error("field '%s' has %zu values (got %zu)", name, s->n * (size_t)comps, count);
    return PG_EINVAL;
  }
  int have = sys_prec ? (s->f64 ? PG_F64 : PG_F32) : PG_F64;
  if (std::string(name) == "acc" || std::string(name) == "drho") have = s->f64 ? PG_F64 : PG_F32;
  if (dtype != have) {
    pg::set_error("asynchronous copies of '%s' need its own precision (dtype %d)", name, have);
    return PG_EINVAL;
  }
  *out = b;
  *bytes = (have == PG_F64 ? 8 : 4) * count;
  return PG_OK;
}

int pg_set_field(pg_system* s, const char* name, const void* host, size_t count, int dtype) {
  PG_TRY(check(s));
  if (!name || (!host && count)) {
    pg::set_error("null name or buffer");
    return PG_EINVAL;
  }
  if (strcmp(name, "rho") != 0) s->stage_pending = false;  // only densities may change between stages
  if (dtype != PG_F32 && dtype != PG_F64) {
    pg::set_error("dtype must be PG_F32 or PG_F64");
    return PG_EINVAL;
  }
  int comps;
  bool sys_prec, writable;
  pg::DevBuf* b = pg::find_field(s, name, &comps, &sys_prec, &writable);
  if (!b) {
    if (count != s->n) {
      pg::set_error("new field '%s' needs n = %zu values (got %zu)", name, s->n, count);
      return PG_EINVAL;
    }
    std::unique_ptr<pg::DevBuf> nb(new pg::DevBuf());
    PG_TRY(nb->ensure(8 * (s->n ? s->n : 1)));
    b = nb.get();
    s->user[name] = std::move(nb);
    comps = 1;
    sys_prec = false;
    writable = true;
  }
  if (!writable) {
    pg::set_error("field '%s' is read-only", name);
    return PG_EINVAL;
  }
  if (count != s->n * (size_t)comps) {
    pg::set_error("field '%s' needs %zu values (got %zu)", name, s->n * (size_t)comps, count);
    return PG_EINVAL;
  }
  const int want = sys_prec ? (s->f64 ? PG_F64 : PG_F32) : PG_F64;
  const size_t eb = want == PG_F64 ? 8 : 4;
  if (dtype == want) {
    if (count) PG_CUDA_TRY(cudaMemcpyAsync(b->p, host, eb * count, cudaMemcpyHostToDevice, s->stream));
  } else {
    std::vector<unsigned char> tmp(eb * count);
    for (size_t i = 0; i < count; ++i) {
      if (want == PG_F64) ((double*)tmp.data())[i] = (double)((const float*)host)[i];
      else ((float*)tmp.data())[i] = (float)((const double*)host)[i];
    }
    if (count) PG_CUDA_TRY(cudaMemcpyAsync(b->p, tmp.data(), eb * count, cudaMemcpyHostToDevice, s->stream));
    PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  }
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  s->nbr_valid = false;
  return PG_OK;
}

int pg_set_field_async(pg_system* s, const char* name, const void* host, size_t count, int dtype) {
  PG_TRY(check(s));
  if (name && strcmp(name, "rho") != 0) s->stage_pending = false;
  pg::DevBuf* b;
  size_t bytes;
  PG_TRY(io_field(s, name, host, count, dtype, true, &b, &bytes));
  pg_system::IoSlot* sl;
  PG_TRY(pg::io_slot(s, name, &sl));
  PG_TRY(sl->stage.ensure(bytes ? bytes : 8));
  PG_CUDA_TRY(cudaStreamWaitEvent(s->io_in, sl->in_free, 0));
  if (bytes) PG_CUDA_TRY(cudaMemcpyAsync(sl->stage.p, host, bytes, cudaMemcpyHostToDevice, s->io_in));
  PG_CUDA_TRY(cudaEventRecord(sl->in_ready, s->io_in));
  sl->in_bytes = bytes;
  sl->pending = true;
  s->nbr_valid = false;
  return PG_OK;
}

int pg_get_field_async(pg_system* s, const char* name, void* host, size_t count, int dtype) {
  PG_TRY(check(s));
  pg::DevBuf* b;
  size_t bytes;
  PG_TRY(io_field(s, name, host, count, dtype, false, &b, &bytes));
  pg_system::IoSlot* sl;
  PG_TRY(pg::io_slot(s, name, &sl));
  PG_TRY(sl->snap.ensure(bytes ? bytes : 8));
  // the snapshot is taken at this point of the compute stream, once its previous copy-out is done
  PG_CUDA_TRY(cudaStreamWaitEvent(s->stream, sl->snap_free, 0));
  if (bytes) PG_CUDA_TRY(cudaMemcpyAsync(sl->snap.p, b->p, bytes, cudaMemcpyDeviceToDevice, s->stream));
  PG_CUDA_TRY(cudaEventRecord(sl->snap_ready, s->stream));
  PG_CUDA_TRY(cudaStreamWaitEvent(s->io_out, sl->snap_ready, 0));
  if (bytes) PG_CUDA_TRY(cudaMemcpyAsync(host, sl->snap.p, bytes, cudaMemcpyDeviceToHost, s->io_out));
  PG_CUDA_TRY(cudaEventRecord(sl->snap_free, s->io_out));
  return PG_OK;
}

int pg_wait_io(pg_system* s) {
  PG_TRY(check(s));
  if (s->io_in) PG_CUDA_TRY(cudaStreamSynchronize(s->io_in));
  if (s->io_out) PG_CUDA_TRY(cudaStreamSynchronize(s->io_out));
  return pg::sync_and_check(s);
}

int pg_get_field(pg_system* s, const char* name, void* host, size_t count, int dtype) {
  PG_TRY(check(s));
  if (!name || (!host && count)) {
    pg::set_error("null name or buffer");
    return PG_EINVAL;
  }
  if (dtype != PG_F32 && dtype != PG_F64) {
    pg::set_error("dtype must be PG_F32 or PG_F64");
    return PG_EINVAL;
  }
  int comps;
  bool sys_prec, writable;
  pg::DevBuf* b = pg::find_field(s, name, &comps, &sys_prec, &writable);
  if (!b) {
    pg::set_error("unknown field '%s' (rates are available after pg_compute_rates)", name);
    return PG_ENOTFOUND;
  }
  if (count != s->n * (size_t)comps) {
    pg::set_error("field '%s' has %zu values (asked for %zu)", name, s->n * (size_t)comps, count);
    return PG_EINVAL;
  }
  int have = sys_prec ? (s->f64 ? PG_F64 : PG_F32) : PG_F64;
  if (std::string(name) == "acc" || std::string(name) == "drho") have = s->f64 ? PG_F64 : PG_F32;
  const size_t eb = have == PG_F64 ? 8 : 4;
  if (dtype == have) {
    if (count) PG_CUDA_TRY(cudaMemcpyAsync(host, b->p, eb * count, cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  } else {
    std::vector<unsigned char> tmp(eb * count);
    if (count) PG_CUDA_TRY(cudaMemcpyAsync(tmp.data(), b->p, eb * count, cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (size_t i = 0; i < count; ++i) {
      if (have == PG_F64) ((float*)host)[i] = (float)((const double*)tmp.data())[i];
      else ((double*)host)[i] = (double)((const float*)tmp.data())[i];
    }
  }
  return PG_OK;
}

int pg_build_neighbors(pg_system* s) {
  PG_TRY(check(s));
  PG_TRY(pg::enqueue_neighbors(s));
  PG_TRY(s->spos.ensure((s->f64 ? 32 : 16) * (s->n ? s->n : 1)));
  NbrArgs a = pg::nbr_args(s);
  PG_TRY(pg::launch_sorted_positions(s->stream, a, s->pos.p, s->spos.p));
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  s->nbr_valid = true;
  return PG_OK;
}

int pg_num_cells(pg_system* s, size_t* n_cells) {
  PG_TRY(check(s));
  if (!n_cells) {
    pg::set_error("null output");
    return PG_EINVAL;
  }
  *n_cells = (size_t)s->ncells;
  return PG_OK;
}

int pg_get_neighbors(pg_system* s, uint32_t* cell_sorted, uint32_t* ids_sorted, uint32_t* cell_start,
                     size_t n_cells_plus_1) {
  PG_TRY(check(s));
  if (!s->nbr_valid) {
    pg::set_error("call pg_build_neighbors first");
    return PG_ESTATE;
  }
  if (cell_start && n_cells_plus_1 != s->ncells + 1) {
    pg::set_error("cell_start needs %llu entries", (unsigned long long)(s->ncells + 1));
    return PG_EINVAL;
  }
  if (cell_sorted && s->n)
    PG_CUDA_TRY(cudaMemcpy(cell_sorted, s->nw.sorted_cell, 4 * s->n, cudaMemcpyDeviceToHost));
  if (ids_sorted && s->n) PG_CUDA_TRY(cudaMemcpy(ids_sorted, s->nw.sorted_id, 4 * s->n, cudaMemcpyDeviceToHost));
  if (cell_start)
    PG_CUDA_TRY(cudaMemcpy(cell_start, s->nw.cell_start.p, 4 * (s->ncells + 1), cudaMemcpyDeviceToHost));
  return PG_OK;
}

int pg_count_neighbors(pg_system* s, uint32_t* counts) {
  PG_TRY(check(s));
  if (!counts && s->n) {
    pg::set_error("null output");
    return PG_EINVAL;
  }
  PG_TRY(pg_build_neighbors(s));
  PG_TRY(s->tmp.ensure(4 * (s->n + 1)));
  NbrArgs a = pg::nbr_args(s);
  PG_TRY(pg::launch_neighbor_counts(s->stream, a, s->tmp.as<uint32_t>()));
  if (s->n) PG_CUDA_TRY(cudaMemcpyAsync(counts, s->tmp.p, 4 * s->n, cudaMemcpyDeviceToHost, s->stream));
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

int pg_get_neighbor_list(pg_system* s, uint64_t* offsets, uint32_t* neighbors, size_t capacity, size_t* total) {
  PG_TRY(check(s));
  if (!offsets) {
    pg::set_error("null offsets");
    return PG_EINVAL;
  }
  PG_TRY(pg_build_neighbors(s));
  const size_t n = s->n;
  PG_TRY(s->tmp.ensure(4 * (n + 1)));
  PG_TRY(s->tmp2.ensure(4 * (n + 1)));
  PG_TRY(s->tmp3.ensure(4 * pg::scan_tmp_words(n)));
  NbrArgs a = pg::nbr_args(s);
  PG_TRY(pg::launch_neighbor_counts(s->stream, a, s->tmp.as<uint32_t>()));
  PG_TRY(pg::launch_exclusive_scan(s->stream, s->tmp.as<uint32_t>(), s->tmp2.as<uint32_t>(), n,
                                   s->tmp3.as<uint32_t>()));
  std::vector<uint32_t> offs32(n + 1);
  PG_CUDA_TRY(cudaMemcpyAsync(offs32.data(), s->tmp2.p, 4 * (n + 1), cudaMemcpyDeviceToHost, s->stream));
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  const size_t tot = offs32[n];
  if (total) *total = tot;
  for (size_t i = 0; i <= n; ++i) offsets[i] = offs32[i];
  if (tot > capacity || (!neighbors && tot)) {
    pg::set_error("neighbour list needs %zu entries (capacity %zu)", tot, capacity);
    return PG_EOVERFLOW;
  }
  pg::DevBuf list;
  PG_TRY(list.ensure(4 * (tot ? tot : 1)));
  PG_TRY(pg::launch_neighbor_list(s->stream, a, s->tmp2.as<uint32_t>(), list.as<uint32_t>()));
  if (tot) PG_CUDA_TRY(cudaMemcpyAsync(neighbors, list.p, 4 * tot, cudaMemcpyDeviceToHost, s->stream));
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

int pg_get_pair_lists(pg_system* s, uint32_t* lengths, uint32_t* entries, size_t capacity) {
  PG_TRY(check(s));
  if (s->model != PG_MODEL_SPH) {
    pg::set_error("pair lists exist for SPH systems only");
    return PG_EINVAL;
  }
  if (!lengths) {
    pg::set_error("null lengths");
    return PG_EINVAL;
  }
  if (s->list_arith < 0 || s->list_arith != s->arith) {
    pg::set_error("no pair lists for the current arithmetic mode yet (run a step or pg_compute_rates)");
    return PG_EINVAL;
  }
  const size_t n = s->n, need = n * (size_t)s->list_cap;
  const size_t stored = (n + pg::kListTile - 1) / pg::kListTile * pg::kListTile * (size_t)s->list_cap;
  if (entries && capacity < need) {
    pg::set_error("pair lists need %zu entries (capacity %zu)", need, capacity);
    return PG_EOVERFLOW;
  }
  PG_TRY(pg::sync_and_check(s));
  if (n) PG_CUDA_TRY(cudaMemcpy(lengths, s->nlen.p, 4 * n, cudaMemcpyDeviceToHost));
  if (entries && need) {  // the device lists are tiled by 32 slots; the caller gets them slot by slot
    std::vector<uint32_t> tiled(stored);
    PG_CUDA_TRY(cudaMemcpy(tiled.data(), s->nlist.p, 4 * stored, cudaMemcpyDeviceToHost));
    const size_t cap = (size_t)s->list_cap, T = pg::kListTile;
    for (size_t k = 0; k < n; ++k)
      for (size_t q = 0; q < cap; ++q) entries[k * cap + q] = tiled[(k / T) * cap * T + q * T + k % T];
  }
  return PG_OK;
}

int pg_gather_sum(pg_system* s, const char* dst, const char* src) {
  PG_TRY(check(s));
  if (!dst || !src) {
    pg::set_error("null field name");
    return PG_EINVAL;
  }
  int cd, cs;
  bool pd, ps, wd, ws;
  pg::DevBuf* bd = pg::find_field(s, dst, &cd, &pd, &wd);
  pg::DevBuf* bs = pg::find_field(s, src, &cs, &ps, &ws);
  if (!bd || !bs) {
    pg::set_error("unknown field '%s'", bd ? src : dst);
    return PG_ENOTFOUND;
  }
  const bool dbl_d = !pd || s->f64, dbl_s = !ps || s->f64;
  if (cd != 1 || cs != 1 || !dbl_d || !dbl_s || !wd) {
    pg::set_error("pg_gather_sum needs writable scalar double fields");
    return PG_EINVAL;
  }
  PG_TRY(pg_build_neighbors(s));
  PG_TRY(s->tmp4.ensure(8 * (s->n ? s->n : 1)));
  PG_TRY(pg::launch_gather_field(s->stream, s->nw.sorted_id, (uint32_t)s->n, bs->as<double>(), s->tmp4.as<double>()));
  NbrArgs a = pg::nbr_args(s);
  PG_TRY(pg::launch_gather_sum(s->stream, a, s->tmp4.as<double>(), bd->as<double>()));
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PG_OK;
}

int pg_compute_rates(pg_system* s) {
  PG_TRY(check(s));
  if (s->model != PG_MODEL_SPH) {
    pg::set_error("pg_compute_rates is for SPH systems");
    return PG_EINVAL;
  }
  const size_t eb = pg::pg_elem_bytes(s);
  const size_t n = s->n ? s->n : 1;
  PG_TRY(s->acc.ensure(eb * n * s->dim));
  PG_TRY(s->drho.ensure(eb * n));
  PG_TRY(pg::enqueue_sph_step(s, true, 0, nullptr));
  PG_TRY(pg::sync_and_check(s));
  s->nbr_valid = false;
  return PG_OK;
}

int pg_step_async(pg_system* s, int nsteps) {
  PG_TRY(check(s));
  if (nsteps < 0) {
    pg::set_error("nsteps < 0");
    return PG_EINVAL;
  }
  for (int i = 0; i < nsteps; ++i) PG_TRY(pg::enqueue_step(s));
  s->nbr_valid = false;
  return PG_OK;
}

int pg_sync(pg_system* s) {
  PG_TRY(check(s));
  return pg::sync_and_check(s);
}

int pg_step(pg_system* s, int nsteps) {
  PG_TRY(pg_step_async(s, nsteps));
  return pg::sync_and_check(s);
}

int pg_step_stage(pg_system* s, int stage) {
  PG_TRY(check(s));
  if (s->model != PG_MODEL_SPH) {
    pg::set_error("pg_step_stage is for SPH systems");
    return PG_EINVAL;
  }
  if (stage == 0) {
    PG_TRY(pg::enqueue_sph_front(s, nullptr));
    s->nbr_valid = false;
    PG_TRY(pg::sync_and_check(s));
    s->stage_pending = true;
    return PG_OK;
  }
  if (stage != 1) {
    pg::set_error("stage must be 0 or 1 (got %d)", stage);
    return PG_EINVAL;
  }
  if (!s->stage_pending) {
    pg::set_error("pg_step_stage(1) needs pg_step_stage(0) first, with no other step, neighbour search or "
                  "field change but rho in between");
    return PG_ESTATE;
  }
  s->stage_pending = false;
  SphArgs a = pg::sph_args(s, 1, false);
  PG_TRY(pg::launch_sph_repack_rho(s->stream, a, s->arith));
  s->launches += 1;
  PG_TRY(pg::enqueue_sph_momentum(s, nullptr));
  return pg::sync_and_check(s);
}

int pg_enable_graph(pg_system* s, int enable) {
  PG_TRY(check(s));
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (!enable) {
    pg::drop_graphs(s);
    s->graph_enabled = false;
    return PG_OK;
  }
  PG_TRY(pg::capture_graphs(s));
  s->graph_enabled = true;
  return PG_OK;
}

int pg_dem_contacts(pg_system* s, long long* contacts) {
  PG_TRY(check(s));
  if (s->model != PG_MODEL_DEM || !contacts) {
    pg::set_error("DEM handle and output required");
    return PG_EINVAL;
  }
  unsigned long long c = 0;
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  PG_CUDA_TRY(cudaMemcpy(&c, s->contacts.p, sizeof(c), cudaMemcpyDeviceToHost));
  *contacts = (long long)c;
  return PG_OK;
}

int pg_dem_get_history(pg_system* s, uint32_t* partner, double* xi, size_t capacity) {
  PG_TRY(check(s));
  if (s->model != PG_MODEL_DEM || capacity != (size_t)s->cfg.contact_capacity) {
    pg::set_error("DEM handle with capacity %d required", s->cfg.contact_capacity);
    return PG_EINVAL;
  }
  const size_t C = capacity;
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (partner && s->n) PG_CUDA_TRY(cudaMemcpy(partner, s->hpid[s->hcur].p, 4 * s->n * C, cudaMemcpyDeviceToHost));
  if (xi && s->n) PG_CUDA_TRY(cudaMemcpy(xi, s->hxi[s->hcur].p, 8 * s->n * C * 3, cudaMemcpyDeviceToHost));
  return PG_OK;
}

int pg_dem_set_history(pg_system* s, const uint32_t* partner, const double* xi, size_t capacity) {
  PG_TRY(check(s));
  if (s->model != PG_MODEL_DEM || capacity != (size_t)s->cfg.contact_capacity || !partner || !xi) {
    pg::set_error("DEM handle with capacity %d and both buffers required", s->cfg.contact_capacity);
    return PG_EINVAL;
  }
  const size_t C = capacity;
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (s->n) {
    // a particle's history ends at its first empty slot; every slot after it is stored empty
    // (no partner, zero spring), the form the contact pass keeps and the oracle produces
    std::vector<uint32_t> p(partner, partner + s->n * C);
    std::vector<double> x(xi, xi + s->n * C * 3);
    for (size_t i = 0; i < s->n; ++i) {
      bool ended = false;
      for (size_t k = 0; k < C; ++k) {
        const size_t o = i * C + k;
        ended = ended || p[o] == 0xFFFFFFFFu;
        if (ended) {
          p[o] = 0xFFFFFFFFu;
          x[3 * o] = x[3 * o + 1] = x[3 * o + 2] = 0.0;
        }
      }
    }
    PG_CUDA_TRY(cudaMemcpy(s->hpid[s->hcur].p, p.data(), 4 * s->n * C, cudaMemcpyHostToDevice));
    PG_CUDA_TRY(cudaMemcpy(s->hxi[s->hcur].p, x.data(), 8 * s->n * C * 3, cudaMemcpyHostToDevice));
  }
  return PG_OK;
}

int pg_timing_enable(pg_system* s, int enable) {
  PG_TRY(check(s));
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  for (cudaEvent_t e : s->ev_pending) s->ev_pool.push_back(e);
  s->ev_pending.clear();
  memset(&s->tacc, 0, sizeof(s->tacc));
  s->timing = enable != 0;
  s->launches = 0;
  return PG_OK;
}

int pg_timing_read(pg_system* s, pg_timing* out) {
  PG_TRY(check(s));
  if (!out) {
    pg::set_error("null output");
    return PG_EINVAL;
  }
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  PG_TRY(pg::timing_collect(s));
  *out = s->tacc;
  out->launches = s->launches;
  return PG_OK;
}

int pg_memory_bytes(pg_system* s, size_t* bytes) {
  PG_TRY(check(s));
  if (!bytes) {
    pg::set_error("null output");
    return PG_EINVAL;
  }
  size_t b = s->nw.bytes();
  const pg::DevBuf* bufs[] = {&s->gridk, &s->sys_of_id, &s->sphk, &s->demk, &s->pos,   &s->vel,     &s->rho,
                              &s->mass,  &s->omega,     &s->radius, &s->acc, &s->drho, &s->spos,    &s->tmp,
                              &s->tmp2,  &s->tmp3,      &s->tmp4,  &s->hpid[0], &s->hpid[1], &s->hxi[0], &s->hxi[1],
                              &s->contacts, &s->err};
  for (const pg::DevBuf* d : bufs) b += d->bytes;
  for (int i = 0; i < 6; ++i) b += s->sorted[i].bytes;
  b += s->nlist.bytes + s->nlen.bytes + s->nresume.bytes + s->fcache.bytes;
  for (auto& kv : s->user) b += kv.second->bytes;
  b += s->adjoint_bytes();
  *bytes = b;
  return PG_OK;
}

int pg_get_info(pg_system* s, pg_info* info) {
  PG_TRY(check(s));
  if (!info) {
    pg::set_error("null output");
    return PG_EINVAL;
  }
  memset(info, 0, sizeof(*info));
  info->n = (long long)s->n;
  info->n_systems = s->nsys;
  info->dim = s->dim;
  info->precision = s->f64 ? PG_F64 : PG_F32;
  info->model = s->model;
  info->arith = s->arith;
  info->n_cells = (long long)s->ncells;
  info->reach = s->grids[0].reach;
  info->pass_grid = s->pass_grid[SPH_MOM];
  info->sort_passes = s->nw.passes;
  for (int d = 0; d < 3; ++d) {
    info->grid_n[d] = s->grids[0].n[d];
    info->grid_lo[d] = s->grids[0].lo[d];
  }
  info->cell_size = s->grids[0].cell;
  info->graph = s->graph_enabled ? 1 : 0;
  info->list_capacity = s->list_cap;
  info->overlap_split = (long long)s->ov_split;
  info->block_size = s->block;
  info->momentum_block = pg::mom_block(s);
  info->particles_per_warp = 32 / pg::sph_pass_lanes(s->arith, pg::SPH_MOM, s->lanes);
  return PG_OK;
}

}  // extern "C"
