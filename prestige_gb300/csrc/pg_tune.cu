// Autotuner of the SPH step: picks the cell-size multiplier, the arithmetic mode and the block
// size of the list-based kernels by timing them on the handle's own particles.
//
// The reference has no tuner (it has no executable backend: prestige/src/codegen/simple_cpu.rs
// returns text).  The knobs change only the schedule, never the method:
//   cell multiplier 1 (27 cells of side 2h) or 1/2 (125 cells of side h): fewer candidates per
//     particle against more rows to walk; the neighbour set is the same, the summation order of
//     the IEEE modes follows the traversal (so results stay within rounding of each other);
//   arithmetic mode (f64: IEEE double or double-word; f32: IEEE single or contracted): a fast
//     mode is accepted only if its rates at the current state are within the mode's tolerance
//     of the IEEE rates (1e-10 normwise for f64, 1e-4 for f32);
//   block size 64, 128 or 256 threads, then the momentum pass's own block size with the rest
//   fixed (it runs alone and shares neighbour records between consecutive slots, so it can
//   prefer larger blocks than the kernels that share the SMs), then the common block size again
//   with the momentum block fixed;
//   particles per warp of the continuity and momentum passes (32, 16 or 8: one, two or four
//   threads per particle, each taking every second or fourth list entry), in the
//   tolerance-based modes only, with the rest fixed.
// The state is restored after every trial and at the end; a graph-enabled handle is re-captured
// with the chosen settings.
#include <cuda_runtime.h>
#include <string.h>

#include <cmath>
#include <vector>

#include "pg_system.cuh"

namespace pg {
namespace {

struct Saved {
  DevBuf pos, vel, rho;
};

int save_state(pg_system* s, Saved& v) {
  const size_t eb = pg_elem_bytes(s), nd = s->n * (size_t)s->dim, n = s->n ? s->n : 1;
  PG_TRY(v.pos.ensure(eb * (nd ? nd : 1)));
  PG_TRY(v.vel.ensure(eb * (nd ? nd : 1)));
  PG_TRY(v.rho.ensure(eb * n));
  if (s->n) {
    PG_CUDA_TRY(cudaMemcpyAsync(v.pos.p, s->pos.p, eb * nd, cudaMemcpyDeviceToDevice, s->stream));
    PG_CUDA_TRY(cudaMemcpyAsync(v.vel.p, s->vel.p, eb * nd, cudaMemcpyDeviceToDevice, s->stream));
    PG_CUDA_TRY(cudaMemcpyAsync(v.rho.p, s->rho.p, eb * s->n, cudaMemcpyDeviceToDevice, s->stream));
  }
  return PG_OK;
}

int restore_state(pg_system* s, const Saved& v) {
  const size_t eb = pg_elem_bytes(s), nd = s->n * (size_t)s->dim;
  if (s->n) {
    PG_CUDA_TRY(cudaMemcpyAsync(s->pos.p, v.pos.p, eb * nd, cudaMemcpyDeviceToDevice, s->stream));
    PG_CUDA_TRY(cudaMemcpyAsync(s->vel.p, v.vel.p, eb * nd, cudaMemcpyDeviceToDevice, s->stream));
    PG_CUDA_TRY(cudaMemcpyAsync(s->rho.p, v.rho.p, eb * s->n, cudaMemcpyDeviceToDevice, s->stream));
  }
  s->nbr_valid = false;
  return PG_OK;
}

// Rates of the current state (acc and drho, id order), as doubles on the host.
int host_rates(pg_system* s, std::vector<double>& out) {
  PG_TRY(pg_compute_rates(s));
  const size_t na = s->n * (size_t)s->dim;
  out.assign(na + s->n, 0.0);
  if (s->f64) {
    PG_TRY(pg_get_field(s, "acc", out.data(), na, PG_F64));
    PG_TRY(pg_get_field(s, "drho", out.data() + na, s->n, PG_F64));
  } else {
    std::vector<float> f(na + s->n);
    PG_TRY(pg_get_field(s, "acc", f.data(), na, PG_F32));
    PG_TRY(pg_get_field(s, "drho", f.data() + na, s->n, PG_F32));
    for (size_t i = 0; i < f.size(); ++i) out[i] = f[i];
  }
  return PG_OK;
}

// max |a - b| / max |b|, separately for the acceleration and density-rate blocks.
double normwise(const std::vector<double>& a, const std::vector<double>& b, size_t na) {
  double worst = 0.0;
  for (int blk = 0; blk < 2; ++blk) {
    const size_t lo = blk ? na : 0, hi = blk ? b.size() : na;
    double num = 0.0, den = 0.0;
    for (size_t i = lo; i < hi; ++i) {
      num = std::fmax(num, std::fabs(a[i] - b[i]));
      den = std::fmax(den, std::fabs(b[i]));
    }
    const double r = den > 0.0 ? num / den : num;
    if (!(r <= worst)) worst = r;  // NaN counts as failing
  }
  return worst;
}

int time_steps(pg_system* s, int steps, double* ms) {
  cudaEvent_t e0, e1;
  PG_CUDA_TRY(cudaEventCreate(&e0));
  PG_CUDA_TRY(cudaEventCreate(&e1));
  int st = PG_OK;
  if (cudaEventRecord(e0, s->stream) != cudaSuccess) st = PG_ECUDA;
  for (int i = 0; i < steps && st == PG_OK; ++i) st = enqueue_step(s);
  if (st == PG_OK && cudaEventRecord(e1, s->stream) != cudaSuccess) st = PG_ECUDA;
  if (st == PG_OK) st = sync_and_check(s);
  float t = 0.f;
  if (st == PG_OK && cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) st = PG_ECUDA;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st == PG_ECUDA) set_error("timing a tuning trial failed");
  *ms = (double)t / (steps > 0 ? steps : 1);
  return st;
}

// Independent FMA chains, eight per thread: throughput of the FMA pipe of type T.
template <class T>
__device__ __forceinline__ T fma_rn(T a, T b, T c);
template <>
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
template <>
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }

constexpr int kChains = 8;

template <class T>
__global__ void fma_chains_kernel(T* out, int iters, T a, T b) {
  T acc[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) acc[c] = (T)(threadIdx.x + c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) acc[c] = fma_rn<T>(acc[c], a, b);
  }
  T sum = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) sum += acc[c];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = sum;
}

// TFLOP/s of the chains (two flops per FMA), timed with events after one warm-up launch.
template <class T>
int time_fma_chains(cudaStream_t st, void* out, int blocks, int threads, int iters, double* tflops) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t err = cudaEventCreate(&e0);
  if (err == cudaSuccess) err = cudaEventCreate(&e1);
  float ms = 0.f;
  if (err == cudaSuccess) {
    fma_chains_kernel<T><<<blocks, threads, 0, st>>>((T*)out, iters / 10, (T)0.999, (T)1e-3);
    cudaEventRecord(e0, st);
    fma_chains_kernel<T><<<blocks, threads, 0, st>>>((T*)out, iters, (T)0.999, (T)1e-3);
    cudaEventRecord(e1, st);
    err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (err != cudaSuccess) {
    set_error("FMA chains: %s", cudaGetErrorString(err));
    return PG_ECUDA;
  }
  *tflops = 2.0 * kChains * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
  return PG_OK;
}

}  // namespace
}  // namespace pg

extern "C" {

int pg_measure_fma_peaks(double* fp64_tflops, double* fp32_tflops) {
  pg::clear_error();
  int dev = 0, sms = 0;
  PG_CUDA_TRY(cudaGetDevice(&dev));
  PG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256;
  cudaStream_t st = nullptr;
  PG_CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  void* out = nullptr;
  cudaError_t err = cudaMalloc(&out, (size_t)blocks * threads * sizeof(double));
  if (err != cudaSuccess) {
    cudaStreamDestroy(st);
    pg::set_error("cudaMalloc: %s", cudaGetErrorString(err));
    return PG_ECUDA;
  }
  double t64 = 0.0, t32 = 0.0;
  int rc = pg::time_fma_chains<double>(st, out, blocks, threads, 2000, &t64);
  if (rc == PG_OK) rc = pg::time_fma_chains<float>(st, out, blocks, threads, 20000, &t32);
  cudaFree(out);
  cudaStreamDestroy(st);
  if (rc != PG_OK) return rc;
  if (fp64_tflops) *fp64_tflops = t64;
  if (fp32_tflops) *fp32_tflops = t32;
  return PG_OK;
}


int pg_set_tuning(pg_system* s, int block, double cell_multiplier, int f64_mode) {
  pg::clear_error();
  if (!s) {
    pg::set_error("null handle");
    return PG_EINVAL;
  }
  const bool graph = s->graph_enabled;
  PG_TRY(pg::retune_sph(s, cell_multiplier, f64_mode, block));
  if (graph) PG_TRY(pg::capture_graphs(s));
  return PG_OK;
}

int pg_set_momentum_block(pg_system* s, int block) {
  pg::clear_error();
  if (!s) {
    pg::set_error("null handle");
    return PG_EINVAL;
  }
  const bool graph = s->graph_enabled;
  PG_TRY(pg::set_momentum_block(s, block));
  if (graph) PG_TRY(pg::capture_graphs(s));
  return PG_OK;
}

int pg_set_particles_per_warp(pg_system* s, int particles_per_warp) {
  pg::clear_error();
  if (!s) {
    pg::set_error("null handle");
    return PG_EINVAL;
  }
  if (particles_per_warp != 32 && particles_per_warp != 16 && particles_per_warp != 8) {
    pg::set_error("particles per warp %d must be 32, 16 or 8", particles_per_warp);
    return PG_EINVAL;
  }
  const bool graph = s->graph_enabled;
  PG_TRY(pg::set_pass_lanes(s, 32 / particles_per_warp));
  if (graph) PG_TRY(pg::capture_graphs(s));
  return PG_OK;
}

int pg_autotune(pg_system* s, int trial_steps, int* best_block, double* best_multiplier, int* best_f64_mode,
                double* best_ms_per_step) {
  pg::clear_error();
  if (!s) {
    pg::set_error("null handle");
    return PG_EINVAL;
  }
  if (s->model != PG_MODEL_SPH) {
    pg::set_error("pg_autotune tunes SPH handles");
    return PG_EINVAL;
  }
  if (trial_steps < 1) {
    pg::set_error("trial_steps must be >= 1");
    return PG_EINVAL;
  }
  PG_CUDA_TRY(cudaStreamSynchronize(s->stream));
  const bool graph = s->graph_enabled;
  const bool timing = s->timing;
  s->graph_enabled = false;
  s->timing = false;
  const double mult0 = s->cfg.cell_multiplier;
  const int mode0 = s->cfg.f64_mode, block0 = s->block;
  pg::Saved saved;
  PG_TRY(pg::save_state(s, saved));

  // reference rates: IEEE mode at the handle's own multiplier
  std::vector<double> ref, got;
  int st = pg::retune_sph(s, mult0, PG_F64_NATIVE, block0);
  if (st == PG_OK) st = pg::restore_state(s, saved);
  if (st == PG_OK) st = pg::host_rates(s, ref);
  const size_t na = s->n * (size_t)s->dim;
  const double tol = s->f64 ? 1e-10 : 1e-4;

  const double mults[2] = {1.0, 0.5};
  const int modes[2] = {PG_F64_NATIVE, PG_F64_FAST};
  const int blocks[3] = {64, 128, 256};
  double best = -1.0;
  double bm = mult0;
  int bmode = mode0, bblock = block0;
  for (int mi = 0; mi < 2 && st == PG_OK; ++mi) {
    for (int oi = 0; oi < 2 && st == PG_OK; ++oi) {
      if (modes[oi] == PG_F64_FAST) {  // accuracy gate, once per (multiplier, mode)
        st = pg::retune_sph(s, mults[mi], modes[oi], 128);
        if (st == PG_OK) st = pg::restore_state(s, saved);
        if (st == PG_OK) st = pg::host_rates(s, got);
        if (st != PG_OK) break;
        if (!(pg::normwise(got, ref, na) <= tol)) continue;
      }
      for (int bi = 0; bi < 3 && st == PG_OK; ++bi) {
        double ms = 0.0;
        st = pg::retune_sph(s, mults[mi], modes[oi], blocks[bi]);
        if (st == PG_OK) st = pg::restore_state(s, saved);
        if (st == PG_OK) st = pg::time_steps(s, 1, &ms);  // warm-up
        if (st == PG_OK) st = pg::restore_state(s, saved);
        if (st == PG_OK) st = pg::time_steps(s, trial_steps, &ms);
        if (st == PG_OK && (best < 0.0 || ms < best)) {
          best = ms;
          bm = mults[mi];
          bmode = modes[oi];
          bblock = blocks[bi];
        }
      }
    }
  }
  // the momentum pass's own block size, with the other settings fixed at the winner
  int bmom = 0;
  if (st == PG_OK) st = pg::retune_sph(s, bm, bmode, bblock);
  double best_mom = -1.0;
  for (int bi = 0; bi < 3 && st == PG_OK; ++bi) {
    double ms = 0.0;
    st = pg::set_momentum_block(s, blocks[bi]);
    if (st == PG_OK) st = pg::restore_state(s, saved);
    if (st == PG_OK) st = pg::time_steps(s, 1, &ms);  // warm-up
    if (st == PG_OK) st = pg::restore_state(s, saved);
    if (st == PG_OK) st = pg::time_steps(s, trial_steps, &ms);
    if (st == PG_OK && (best_mom < 0.0 || ms < best_mom)) {
      best_mom = ms;
      bmom = blocks[bi];
    }
  }
  if (st == PG_OK && best_mom >= 0.0) best = best_mom;
  // the common block size again, with the momentum pass's block fixed (the first search ran the
  // momentum pass at the common block size, which biases it towards the momentum pass's choice)
  for (int bi = 0; bi < 3 && st == PG_OK; ++bi) {
    if (blocks[bi] == bblock) continue;
    double ms = 0.0;
    st = pg::retune_sph(s, bm, bmode, blocks[bi]);
    if (st == PG_OK) st = pg::set_momentum_block(s, bmom);
    if (st == PG_OK) st = pg::restore_state(s, saved);
    if (st == PG_OK) st = pg::time_steps(s, 1, &ms);  // warm-up
    if (st == PG_OK) st = pg::restore_state(s, saved);
    if (st == PG_OK) st = pg::time_steps(s, trial_steps, &ms);
    if (st == PG_OK && ms < best) {
      best = ms;
      bblock = blocks[bi];
    }
  }
  // particles per warp of the pair passes (tolerance-based modes only), the rest fixed
  int blanes = 1;
  if (st == PG_OK) st = pg::retune_sph(s, bm, bmode, bblock);
  if (st == PG_OK) st = pg::set_momentum_block(s, bmom);
  const int lanes[2] = {2, 4};
  for (int li = 0; li < 2 && st == PG_OK && pg::sph_pass_lanes(s->arith, pg::SPH_MOM, 2) > 1; ++li) {
    double ms = 0.0;
    st = pg::set_pass_lanes(s, lanes[li]);
    if (st == PG_OK) st = pg::restore_state(s, saved);
    if (st == PG_OK) st = pg::time_steps(s, 1, &ms);  // warm-up
    if (st == PG_OK) st = pg::restore_state(s, saved);
    if (st == PG_OK) st = pg::time_steps(s, trial_steps, &ms);
    if (st == PG_OK && ms < best) {
      best = ms;
      blanes = lanes[li];
    }
  }
  // apply the winner (or, after a failure, the original settings) and restore the state
  int st_apply = pg::retune_sph(s, st == PG_OK ? bm : mult0, st == PG_OK ? bmode : mode0,
                                st == PG_OK ? bblock : block0);
  if (st == PG_OK && st_apply == PG_OK) st_apply = pg::set_momentum_block(s, bmom);
  if (st == PG_OK && st_apply == PG_OK) st_apply = pg::set_pass_lanes(s, blanes);
  const int st_restore = pg::restore_state(s, saved);
  s->timing = timing;
  if (st == PG_OK) st = st_apply;
  if (st == PG_OK) st = st_restore;
  if (st == PG_OK) st = pg::sync_and_check(s);
  if (st == PG_OK && graph) {
    st = pg::capture_graphs(s);
    s->graph_enabled = st == PG_OK;
  }
  if (st != PG_OK) return st;
  if (best_block) *best_block = bblock;
  if (best_multiplier) *best_multiplier = bm;
  if (best_f64_mode) *best_f64_mode = bmode;
  if (best_ms_per_step) *best_ms_per_step = best;
  return PG_OK;
}

}  // extern "C"
