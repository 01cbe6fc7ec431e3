// Cell hash, neighbour counts / CSR lists and the eq1 gather of the reference.
//
// The reference's only equation is `force[i] += mass[j]` (prestige/src/lib.rs:7-12), run by
// the generated loop `for i in 0..n { for j in 0..n { ... } }`
// (prestige/src/codegen/simple_cpu.rs:7-8).  launch_gather_sum evaluates that body with j
// over the neighbour set {j : |x_i - x_j| < support} (j == i included), in the oracle's
// traversal order, so integer-valued sums are exact and every sum is bit-exact.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include <cmath>

#include "pg_arith.cuh"
#include "pg_internal.cuh"
#include "pg_kernels.cuh"

namespace pg {

// ---------------------------------------------------------------------------------------
// Errors and buffers.
// ---------------------------------------------------------------------------------------
static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
void clear_error() { g_err[0] = 0; }
const char* last_error() { return g_err; }

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

int DevBuf::ensure(size_t nbytes) {
  if (nbytes <= bytes && p) return PG_OK;
  release();
  if (nbytes == 0) nbytes = 16;
  cudaError_t e = cudaMalloc(&p, nbytes);
  if (e != cudaSuccess) {
    p = nullptr;
    cudaGetLastError();
    set_error("cudaMalloc(%zu bytes) failed: %s", nbytes, cudaGetErrorString(e));
    return PG_ENOMEM;
  }
  bytes = nbytes;
  return PG_OK;
}

// ---------------------------------------------------------------------------------------
// Grid (same formulas as the oracle's make_grid).
// ---------------------------------------------------------------------------------------
int make_grid(int dim, const double lo[3], const double hi[3], double support, double mult, Grid* g) {
  if (!(support > 0.0) || !(mult > 0.0) || !std::isfinite(support) || !std::isfinite(mult)) {
    set_error("grid: support (%g) and cell multiplier (%g) must be positive", support, mult);
    return PG_EINVAL;
  }
  g->dim = dim;
  g->support = support;
  g->cell = mult * support * (1.0 + 0x1p-20);
  g->inv = 1.0 / g->cell;
  uint64_t total = 1;
  for (int d = 0; d < 3; ++d) {
    if (d < dim) {
      if (!(hi[d] > lo[d]) || !std::isfinite(lo[d]) || !std::isfinite(hi[d])) {
        set_error("grid: domain_hi[%d] must exceed domain_lo[%d]", d, d);
        return PG_EINVAL;
      }
      g->lo[d] = lo[d];
      const double cells = std::ceil((hi[d] - lo[d]) / g->cell);
      if (cells > 2.0e9) {
        set_error("grid: %g cells along axis %d", cells, d);
        return PG_EINVAL;
      }
      g->n[d] = cells < 1.0 ? 1 : (int)cells;
    } else {
      g->lo[d] = 0.0;
      g->n[d] = 1;
    }
    total *= (uint64_t)g->n[d];
  }
  if (total >= 0xFFFFFFF0ull) {
    set_error("grid: %llu cells exceed the 32-bit cell index", (unsigned long long)total);
    return PG_EINVAL;
  }
  g->reach = (int)std::ceil(support / g->cell);
  return PG_OK;
}

GridK grid_k(const Grid& g, uint32_t cell_base) {
  GridK k;
  for (int d = 0; d < 3; ++d) {
    k.lo[d] = g.lo[d];
    k.lof[d] = (float)g.lo[d];
  }
  k.inv = 1.0 / g.cell;
  k.invf = (float)(1.0 / g.cell);
  k.support = g.support;
  k.support_f = (float)g.support;
  k.nx = g.n[0];
  k.ny = g.n[1];
  k.nz = g.n[2];
  k.reach = g.reach;
  k.dim = g.dim;
  k.cell_base = cell_base;
  return k;
}

namespace {

template <class R> struct NbrV4;
template <> struct NbrV4<double> { typedef double4_32a T; };
template <> struct NbrV4<float> { typedef float4 T; };

__device__ __forceinline__ int cell_coord_d(double x, double lo, double inv, int n) {
  const double t = __dmul_rn(__dsub_rn(x, lo), inv);
  if (!(t >= 0.0)) return 0;
  if (t >= (double)n) return n - 1;
  return (int)t;
}

// cell_coord_d's result without FP64 work in nearly every case (GB300 runs FP64 at 1/64 of the
// FP32 rate): t = (x - lo) * inv in FP32 from the FP32 copies, with a bound E on its distance
// from the f64 t (8u (|x| + |lo|) inv + 8u |t|, twice the first-order error of the FP32 copies
// and operations).  When [t - E, t + E] lies inside one cell, or entirely below 0 or above n,
// that decides the clamped floor; otherwise (near a cell boundary, NaN) the f64 formula runs.
// The f64 formula, out of line: only particles near a cell boundary run it.
__device__ __noinline__ int cell_coord_d_call(double x, double lo, double inv, int n) {
  return cell_coord_d(x, lo, inv, n);
}

__device__ __forceinline__ int cell_coord_fast(double x, double lo, float lof, double inv, float invf, int n) {
  float xf, xl;
  df_split_fast(x, &xf, &xl);
  const float t = (xf - lof) * invf;
  const float E = 4.76837158203125e-07f * ((fabsf(xf) + fabsf(lof)) * invf + fabsf(t));
  const float a = t - E, b = t + E;
  if (b < 0.f) return 0;
  if (a >= (float)n) return n - 1;
  if (a >= 0.f && b < (float)n) {
    const int ia = (int)a;
    if (ia == (int)b) return ia;
  }
  return cell_coord_d_call(x, lo, inv, n);
}

__device__ __forceinline__ int cell_coord_f(float x, float lo, float inv, int n) {
  const float t = __fmul_rn(__fsub_rn(x, lo), inv);
  if (!(t >= 0.f)) return 0;
  if (t >= (float)n) return n - 1;
  return (int)t;
}

// Cell key and id of every particle.  MIN: also the minimum position per system and dimension
// (posmin[3 sys + d]).  A single system: block reduction, one atomicMin per block and dimension
// (blockDim.x == 256).  A batch: warp reduction where the warp's particles belong to one system
// (ids are contiguous per system, so all warps but those at a system boundary), else one
// atomicMin per particle.
template <class R, int DIM, bool MIN>
__global__ void hash_kernel(const GridK* __restrict__ grid, const uint32_t* __restrict__ sys_of_id,
                            const R* __restrict__ pos, uint32_t n, uint32_t* __restrict__ keys,
                            uint32_t* __restrict__ vals, unsigned long long* __restrict__ posmin) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long m[3] = {~0ull, ~0ull, ~0ull};
  if (i < n) {
    const GridK& g = grid[sys_of_id ? sys_of_id[i] : 0u];
    int c[3] = {0, 0, 0};
    const int nn[3] = {g.nx, g.ny, g.nz};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const R x = pos[(size_t)i * DIM + d];
      if (sizeof(R) == 8) c[d] = cell_coord_fast((double)x, g.lo[d], g.lof[d], g.inv, g.invf, nn[d]);
      else c[d] = cell_coord_f((float)x, g.lof[d], g.invf, nn[d]);
      if (MIN) m[d] = ordered_code((double)x);
    }
    keys[i] = g.cell_base + ((uint32_t)c[2] * (uint32_t)g.ny + (uint32_t)c[1]) * (uint32_t)g.nx + (uint32_t)c[0];
    vals[i] = i;
  }
  if (MIN && sys_of_id) {
    const uint32_t s = i < n ? sys_of_id[i] : 0xffffffffu;
    const uint32_t s0 = __shfl_sync(0xffffffffu, s, 0);
    if (__all_sync(0xffffffffu, s == s0)) {
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        for (int o = 16; o; o >>= 1) m[d] = min(m[d], __shfl_down_sync(0xffffffffu, m[d], o));
        if ((threadIdx.x & 31) == 0 && s0 != 0xffffffffu) atomicMin(posmin + 3 * (size_t)s0 + d, m[d]);
      }
    } else if (i < n) {
#pragma unroll
      for (int d = 0; d < DIM; ++d) atomicMin(posmin + 3 * (size_t)s + d, m[d]);
    }
  } else if (MIN) {
    __shared__ unsigned long long part[DIM][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      for (int o = 16; o; o >>= 1) m[d] = min(m[d], __shfl_down_sync(0xffffffffu, m[d], o));
      if (lane == 0) part[d][warp] = m[d];
    }
    __syncthreads();
    if (threadIdx.x < DIM) {
      unsigned long long v = part[threadIdx.x][0];
      for (int w = 1; w < 8; ++w) v = min(v, part[threadIdx.x][w]);
      atomicMin(posmin + threadIdx.x, v);
    }
  }
}

template <class R, int DIM>
__global__ void sorted_positions_kernel(NbrArgs a, const R* __restrict__ pos, typename NbrV4<R>::T* spos) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const uint32_t id = a.sorted_id[k];
  typename NbrV4<R>::T p;
  p.x = pos[(size_t)id * DIM];
  p.y = pos[(size_t)id * DIM + 1];
  p.z = DIM == 3 ? pos[(size_t)id * DIM + 2] : R(0);
  p.w = R(0);
  spos[k] = p;
}

// r^2 < support^2 in the system precision, oracle order dx*dx + dy*dy (+ dz*dz).
template <class R, int DIM>
__device__ __forceinline__ bool within(const typename NbrV4<R>::T& a, const typename NbrV4<R>::T& b, R s2) {
  if (sizeof(R) == 8) {
    const double d0 = __dsub_rn(a.x, b.x), d1 = __dsub_rn(a.y, b.y);
    double r2 = __dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1));
    if (DIM == 3) {
      const double d2 = __dsub_rn(a.z, b.z);
      r2 = __dadd_rn(r2, __dmul_rn(d2, d2));
    }
    return r2 < (double)s2;
  } else {
    const float d0 = __fsub_rn(a.x, b.x), d1 = __fsub_rn(a.y, b.y);
    float r2 = __fadd_rn(__fmul_rn(d0, d0), __fmul_rn(d1, d1));
    if (DIM == 3) {
      const float d2 = __fsub_rn(a.z, b.z);
      r2 = __fadd_rn(r2, __fmul_rn(d2, d2));
    }
    return r2 < (float)s2;
  }
}

// Visits every candidate slot of slot k's neighbour cells in traversal order:
// rows z then y ascending, slots ascending within a row.
template <class Fn>
__device__ __forceinline__ void for_each_candidate(const NbrArgs& a, const GridK& g, uint32_t k, Fn&& fn) {
  const uint32_t c = a.sorted_cell[k] - g.cell_base;
  const int cx = (int)(c % (uint32_t)g.nx);
  const int cy = (int)((c / (uint32_t)g.nx) % (uint32_t)g.ny);
  const int cz = (int)(c / ((uint32_t)g.nx * (uint32_t)g.ny));
  const int R = g.reach;
  const int RZ = g.dim == 3 ? R : 0;
  const int x0 = max(cx - R, 0), x1 = min(cx + R, g.nx - 1);
  for (int dz = -RZ; dz <= RZ; ++dz) {
    const int z = cz + dz;
    if (z < 0 || z >= g.nz) continue;
    for (int dy = -R; dy <= R; ++dy) {
      const int y = cy + dy;
      if (y < 0 || y >= g.ny) continue;
      const uint32_t rb = g.cell_base + ((uint32_t)z * g.ny + (uint32_t)y) * g.nx;
      const uint32_t s = a.cell_start[rb + x0], e = a.cell_start[rb + x1 + 1];
      for (uint32_t t = s; t < e; ++t) fn(t);
    }
  }
}

template <class R>
__device__ __forceinline__ R support2(const GridK& g) {
  if (sizeof(R) == 8) return (R)__dmul_rn(g.support, g.support);
  return (R)__fmul_rn(g.support_f, g.support_f);
}

template <class R, int DIM>
__global__ void neighbor_counts_kernel(NbrArgs a, uint32_t* __restrict__ counts) {
  typedef typename NbrV4<R>::T V;
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const uint32_t id = a.sorted_id[k];
  const GridK& g = a.grid[a.sys_of_id ? a.sys_of_id[id] : 0u];
  const V* sp = (const V*)a.spos;
  const V pi = sp[k];
  const R s2 = support2<R>(g);
  uint32_t cnt = 0;
  for_each_candidate(a, g, k, [&](uint32_t t) {
    if (within<R, DIM>(pi, sp[t], s2)) ++cnt;
  });
  counts[id] = cnt;
}

template <class R, int DIM>
__global__ void neighbor_list_kernel(NbrArgs a, const uint32_t* __restrict__ offs, uint32_t* __restrict__ nbr) {
  typedef typename NbrV4<R>::T V;
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const uint32_t id = a.sorted_id[k];
  const GridK& g = a.grid[a.sys_of_id ? a.sys_of_id[id] : 0u];
  const V* sp = (const V*)a.spos;
  const V pi = sp[k];
  const R s2 = support2<R>(g);
  uint32_t o = offs[id];
  for_each_candidate(a, g, k, [&](uint32_t t) {
    if (within<R, DIM>(pi, sp[t], s2)) nbr[o++] = a.sorted_id[t];
  });
}

// dst[i] = dst[i] + src[j] for each neighbour j in traversal order (IEEE double adds).
template <class R, int DIM>
__global__ void gather_sum_kernel(NbrArgs a, const double* __restrict__ src_sorted, double* __restrict__ dst) {
  typedef typename NbrV4<R>::T V;
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const uint32_t id = a.sorted_id[k];
  const GridK& g = a.grid[a.sys_of_id ? a.sys_of_id[id] : 0u];
  const V* sp = (const V*)a.spos;
  const V pi = sp[k];
  const R s2 = support2<R>(g);
  double acc = dst[id];
  for_each_candidate(a, g, k, [&](uint32_t t) {
    if (within<R, DIM>(pi, sp[t], s2)) acc = __dadd_rn(acc, src_sorted[t]);
  });
  dst[id] = acc;
}

__global__ void gather_field_kernel(const uint32_t* __restrict__ sorted_id, uint32_t n, const double* __restrict__ src,
                                    double* __restrict__ out) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = src[sorted_id[k]];
}

inline unsigned blocks_for(size_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

int launch_hash(cudaStream_t st, const GridK* grid_dev, const uint32_t* sys_of_id, int f64, int dim, const void* pos,
                size_t n, uint32_t* keys, uint32_t* vals, unsigned long long* posmin) {
  if (n == 0) return PG_OK;
  const unsigned b = blocks_for(n, 256);
  const uint32_t m = (uint32_t)n;
  if (f64 && posmin) {
    if (dim == 2) hash_kernel<double, 2, true><<<b, 256, 0, st>>>(grid_dev, sys_of_id, (const double*)pos, m, keys, vals, posmin);
    else hash_kernel<double, 3, true><<<b, 256, 0, st>>>(grid_dev, sys_of_id, (const double*)pos, m, keys, vals, posmin);
  } else if (f64) {
    if (dim == 2) hash_kernel<double, 2, false><<<b, 256, 0, st>>>(grid_dev, sys_of_id, (const double*)pos, m, keys, vals, nullptr);
    else hash_kernel<double, 3, false><<<b, 256, 0, st>>>(grid_dev, sys_of_id, (const double*)pos, m, keys, vals, nullptr);
  } else {
    if (dim == 2) hash_kernel<float, 2, false><<<b, 256, 0, st>>>(grid_dev, sys_of_id, (const float*)pos, m, keys, vals, nullptr);
    else hash_kernel<float, 3, false><<<b, 256, 0, st>>>(grid_dev, sys_of_id, (const float*)pos, m, keys, vals, nullptr);
  }
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

int launch_sorted_positions(cudaStream_t st, const NbrArgs& a, const void* pos, void* spos) {
  if (a.n == 0) return PG_OK;
  const unsigned b = blocks_for(a.n, 256);
  if (a.f64) {
    if (a.dim == 2) sorted_positions_kernel<double, 2><<<b, 256, 0, st>>>(a, (const double*)pos, (double4_32a*)spos);
    else sorted_positions_kernel<double, 3><<<b, 256, 0, st>>>(a, (const double*)pos, (double4_32a*)spos);
  } else {
    if (a.dim == 2) sorted_positions_kernel<float, 2><<<b, 256, 0, st>>>(a, (const float*)pos, (float4*)spos);
    else sorted_positions_kernel<float, 3><<<b, 256, 0, st>>>(a, (const float*)pos, (float4*)spos);
  }
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

#define PG_DISPATCH_RD(a, KERNEL, ...)                                                            \
  do {                                                                                            \
    const unsigned b_ = blocks_for((a).n, 128);                                                   \
    if ((a).f64) {                                                                                \
      if ((a).dim == 2) KERNEL<double, 2><<<b_, 128, 0, st>>>(__VA_ARGS__);                       \
      else KERNEL<double, 3><<<b_, 128, 0, st>>>(__VA_ARGS__);                                    \
    } else {                                                                                      \
      if ((a).dim == 2) KERNEL<float, 2><<<b_, 128, 0, st>>>(__VA_ARGS__);                        \
      else KERNEL<float, 3><<<b_, 128, 0, st>>>(__VA_ARGS__);                                     \
    }                                                                                             \
  } while (0)

int launch_neighbor_counts(cudaStream_t st, const NbrArgs& a, uint32_t* counts_by_id) {
  if (a.n == 0) return PG_OK;
  PG_DISPATCH_RD(a, neighbor_counts_kernel, a, counts_by_id);
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

int launch_neighbor_list(cudaStream_t st, const NbrArgs& a, const uint32_t* offs_by_id, uint32_t* nbr) {
  if (a.n == 0) return PG_OK;
  PG_DISPATCH_RD(a, neighbor_list_kernel, a, offs_by_id, nbr);
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

int launch_gather_sum(cudaStream_t st, const NbrArgs& a, const double* src_sorted, double* dst_by_id) {
  if (a.n == 0) return PG_OK;
  PG_DISPATCH_RD(a, gather_sum_kernel, a, src_sorted, dst_by_id);
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

int launch_gather_field(cudaStream_t st, const uint32_t* sorted_id, uint32_t n, const double* src, double* out) {
  if (n == 0) return PG_OK;
  gather_field_kernel<<<blocks_for(n, 256), 256, 0, st>>>(sorted_id, n, src, out);
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

}  // namespace pg
