// The SPH pair-pass skeleton shared by the forward pass (pg_sph.cu) and the adjoint pass
// (pg_adjoint.cu): one thread per target slot, a two-phase candidate walk over the neighbour
// rows (cheap FP32 filter into a per-thread hit list in shared memory, then the exact test and
// the pair terms of a `Pairs` policy over the listed hits), and the Tait pressure term.
//
// A `Pairs` policy provides
//   begin(args, system, slot)   load the target's data
//   pair(slot_j)                one candidate that passed the filter (repeats the exact test)
//   finish(args, system, id, k) write the target's results (id order; k = its slot)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pg_arith.cuh"
#include "pg_internal.cuh"
#include "pg_kernels.cuh"

namespace pg {
namespace sphpass {

constexpr int kHitCap = 32;
constexpr unsigned kFull = 0xffffffffu;

template <class R> struct V4;
template <> struct V4<double> { typedef double4_32a T; };
template <> struct V4<float> { typedef float4 T; };

template <class R> __device__ __forceinline__ const SphC<R>& consts(const SphK& K);
template <> __device__ __forceinline__ const SphC<double>& consts<double>(const SphK& K) { return K.d; }
template <> __device__ __forceinline__ const SphC<float>& consts<float>(const SphK& K) { return K.f; }

// p / rho^2 with p = B((rho/rho0)^gamma - 1), operation order of the oracle's tait_pterm.
template <class Ops>
__device__ __forceinline__ typename Ops::R tait_pterm(const SphC<typename Ops::R>& c, int gamma,
                                                      typename Ops::R rho) {
  typedef typename Ops::R R;
  const R rr = Ops::mul(rho, c.inv_rho0);
  R pw = rr;
  for (int e = 1; e < gamma; ++e) pw = Ops::mul(pw, rr);
  const R p = Ops::mul(c.B, Ops::sub(pw, R(1)));
  return Ops::div(p, Ops::mul(rho, rho));
}

__device__ __forceinline__ uint32_t sys_of_slot(const SphArgs& a, uint32_t id) {
  return a.sys_of_id ? a.sys_of_id[id] : 0u;
}

// ---------------------------------------------------------------------------------------
// Shared pieces of the candidate walk.
// ---------------------------------------------------------------------------------------
struct Target {
  uint32_t k, id;
  bool live;
  int cx, cy, cz, x0, x1;
};

__device__ __forceinline__ Target target_of(const SphArgs& a, uint32_t k0, const SphK** Kp, int R) {
  Target T;
  T.live = k0 < a.n;
  T.k = T.live ? k0 : a.n - 1;
  T.id = a.sorted_id[T.k];
  const SphK& K = a.sys[sys_of_slot(a, T.id)];
  *Kp = &K;
  const GridK& g = K.g;
  const uint32_t c = a.sorted_cell[T.k] - g.cell_base;
  T.cx = (int)(c % (uint32_t)g.nx);
  T.cy = (int)((c / (uint32_t)g.nx) % (uint32_t)g.ny);
  T.cz = (int)(c / ((uint32_t)g.nx * (uint32_t)g.ny));
  T.x0 = max(T.cx - R, 0);
  T.x1 = min(T.cx + R, g.nx - 1);
  return T;
}

// FP32 threshold on r^2.  EXACT_PF (f32 systems): the exact test.  Otherwise a conservative
// bound: |x_j - x_i| < 2h in f64  =>  the FP32 r^2 below is < thr (rounding of positions to
// float and of the FP32 arithmetic bounded with a generous factor).
template <bool EXACT_PF>
__device__ __forceinline__ float prefilter_threshold(const SphK& K, const float4& pi) {
  if (EXACT_PF) return K.f.four_h2;
  const float M = fmaxf(fmaxf(fabsf(pi.x), fabsf(pi.y)), fabsf(pi.z)) + K.two_h_f;
  const float delta = 2.384185791015625e-07f * (2.f * M + K.two_h_f);  // 4u (2M + 2h)
  const float rr = K.two_h_f + 2.f * delta;
  return rr * rr * 1.0000153f;
}

template <int DIM, bool EXACT_PF>
__device__ __forceinline__ bool prefilter_hit(const float4& pi, const float4& pj, float thr) {
  if (EXACT_PF) {
    const float d0 = __fsub_rn(pi.x, pj.x), d1 = __fsub_rn(pi.y, pj.y);
    float r2 = __fadd_rn(__fmul_rn(d0, d0), __fmul_rn(d1, d1));
    if (DIM == 3) {
      const float d2 = __fsub_rn(pi.z, pj.z);
      r2 = __fadd_rn(r2, __fmul_rn(d2, d2));
    }
    return r2 < thr && r2 > 0.f;
  }
  const float d0 = pi.x - pj.x, d1 = pi.y - pj.y;
  float r2 = fmaf(d1, d1, d0 * d0);
  if (DIM == 3) {
    const float d2 = pi.z - pj.z;
    r2 = fmaf(d2, d2, r2);
  }
  return r2 < thr;
}

// ---------------------------------------------------------------------------------------
// The two-phase pass (candidate walk and pair terms in one kernel).  PF: the FP32 position
// array tested in phase 1 (float4 x,y,z per slot).
// ---------------------------------------------------------------------------------------
template <class Pairs, int DIM, bool EXACT_PF>
__global__ void __launch_bounds__(kSphThreads) sph_pass_kernel(SphArgs a, int pf_index) {
  __shared__ uint32_t hits[kHitCap][kSphThreads];
  const int tid = threadIdx.x;
  const float4* __restrict__ PF = (const float4*)a.s[pf_index];
  const uint32_t* __restrict__ start = a.cell_start;
  const int R = a.reach;
  const int RZ = DIM == 3 ? R : 0;
  const int side = 2 * R + 1;
  const int nrows = side * (2 * RZ + 1);
  const uint32_t ntiles = (a.n + kSphThreads - 1) / kSphThreads;

  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const SphK* Kp;
    const Target T = target_of(a, tile * kSphThreads + tid, &Kp, R);
    const SphK& K = *Kp;
    const GridK& g = K.g;

    Pairs P;
    P.begin(a, K, T.k);
    const float4 pi = PF[T.k];
    const float thr = prefilter_threshold<EXACT_PF>(K, pi);

    int nh = 0;
    int row = 0;
    uint32_t t = 0, e = 0;
    while (true) {
      // advance this lane to its next candidate (rows z, y ascending)
      while (t >= e && row < nrows) {
        const int dz = row / side - RZ, dy = row % side - R;
        ++row;
        const int z = T.cz + dz, y = T.cy + dy;
        if (!T.live || z < 0 || z >= g.nz || y < 0 || y >= g.ny) continue;
        const uint32_t rb = g.cell_base + ((uint32_t)z * g.ny + (uint32_t)y) * g.nx;
        t = start[rb + T.x0];
        e = start[rb + T.x1 + 1];
      }
      const bool has = t < e;
      if (has) {
        if (prefilter_hit<DIM, EXACT_PF>(pi, PF[t], thr)) hits[nh++][tid] = t;
        ++t;
      }
      const bool done = !__any_sync(kFull, has);
      if (done || __any_sync(kFull, nh == kHitCap)) {
        for (int h = 0; __any_sync(kFull, h < nh); ++h)
          if (h < nh) P.pair(hits[h][tid]);
        nh = 0;
        if (done) break;
      }
    }
    if (T.live) P.finish(a, K, T.id, T.k);
  }
}

// ---------------------------------------------------------------------------------------
// Neighbour lists.  sph_list_kernel walks the candidates of every slot once per step (the
// same concatenated walk and FP32 prefilter as above) and writes the passing slots, in
// traversal order, to nlist[k * cap ...]; nlen[k] = number of passing slots (may exceed cap).
// When the list fills, nresume[2k], [2k+1] = (row, slot) of the first passing candidate that
// did not fit, so the pair passes can continue the walk from there.
// ---------------------------------------------------------------------------------------
template <int DIM, bool EXACT_PF>
__global__ void __launch_bounds__(kSphMaxThreads) sph_list_kernel(SphArgs a, int pf_index) {
  const int tid = threadIdx.x;
  const float4* __restrict__ PF = (const float4*)a.s[pf_index];
  const uint32_t* __restrict__ start = a.cell_start;
  const int R = a.reach;
  const int RZ = DIM == 3 ? R : 0;
  const int side = 2 * R + 1;
  const int nrows = side * (2 * RZ + 1);
  const uint32_t cap = a.cap;
  const uint32_t bs = blockDim.x;
  const uint32_t ntiles = (a.n + bs - 1) / bs;

  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const SphK* Kp;
    const Target T = target_of(a, tile * bs + tid, &Kp, R);
    const SphK& K = *Kp;
    const GridK& g = K.g;
    const float4 pi = PF[T.k];
    const float thr = prefilter_threshold<EXACT_PF>(K, pi);
    uint32_t* __restrict__ my = a.nlist + (size_t)T.k * cap;
    uint32_t cnt = 0;
    int row = 0;
    uint32_t t = 0, e = 0;
    while (true) {
      while (t >= e && row < nrows) {
        const int dz = row / side - RZ, dy = row % side - R;
        ++row;
        const int z = T.cz + dz, y = T.cy + dy;
        if (!T.live || z < 0 || z >= g.nz || y < 0 || y >= g.ny) continue;
        const uint32_t rb = g.cell_base + ((uint32_t)z * g.ny + (uint32_t)y) * g.nx;
        t = start[rb + T.x0];
        e = start[rb + T.x1 + 1];
      }
      if (!__any_sync(kFull, t < e)) break;
      if (t < e) {
        if (prefilter_hit<DIM, EXACT_PF>(pi, PF[t], thr)) {
          if (cnt < cap) {
            my[cnt] = t;
          } else if (cnt == cap) {
            a.nresume[2 * (size_t)T.k] = (uint32_t)(row - 1);
            a.nresume[2 * (size_t)T.k + 1] = t;
          }
          ++cnt;
        }
        ++t;
      }
    }
    if (T.live) a.nlen[T.k] = cnt;
  }
}

// Pair pass over the lists of sph_list_kernel (any block size up to kSphMaxThreads, a
// multiple of 32).  Lanes step through their lists together;
// a list that overflowed is followed by the rest of the walk from its resume point.
template <class Pairs, int DIM, bool EXACT_PF>
__global__ void __launch_bounds__(kSphMaxThreads) sph_list_pass_kernel(SphArgs a, int pf_index) {
  const int tid = threadIdx.x;
  const uint32_t cap = a.cap;
  const uint32_t bs = blockDim.x;
  const uint32_t ntiles = (a.n + bs - 1) / bs;
  for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint32_t k0 = tile * bs + tid;
    const bool live = k0 < a.n;
    const uint32_t k = live ? k0 : a.n - 1;
    const uint32_t id = a.sorted_id[k];
    const SphK& K = a.sys[sys_of_slot(a, id)];
    Pairs P;
    P.begin(a, K, k);
    const uint32_t cnt = live ? a.nlen[k] : 0u;
    const uint32_t L = min(cnt, cap);
    const uint32_t* __restrict__ my = a.nlist + (size_t)k * cap;
    for (uint32_t q = 0; q < L; ++q) P.pair(my[q]);
    if (cnt > cap) {
      // rare: continue the candidate walk where the list stopped
      const float4* __restrict__ PF = (const float4*)a.s[pf_index];
      const SphK* Kp;
      const Target T = target_of(a, k0, &Kp, a.reach);
      const GridK& g = K.g;
      const int R = a.reach, RZ = DIM == 3 ? R : 0, side = 2 * R + 1, nrows = side * (2 * RZ + 1);
      const float4 pi = PF[k];
      const float thr = prefilter_threshold<EXACT_PF>(K, pi);
      const int row0 = (int)a.nresume[2 * (size_t)k];
      const uint32_t t0 = a.nresume[2 * (size_t)k + 1];
      for (int row = row0; row < nrows; ++row) {
        const int z = T.cz + row / side - RZ, y = T.cy + row % side - R;
        if (z < 0 || z >= g.nz || y < 0 || y >= g.ny) continue;
        const uint32_t rb = g.cell_base + ((uint32_t)z * g.ny + (uint32_t)y) * g.nx;
        const uint32_t e = a.cell_start[rb + T.x1 + 1];
        for (uint32_t t = row == row0 ? t0 : a.cell_start[rb + T.x0]; t < e; ++t)
          if (prefilter_hit<DIM, EXACT_PF>(pi, PF[t], thr)) P.pair(t);
      }
    }
    if (live) P.finish(a, K, id, k);
  }
}

}  // namespace sphpass
}  // namespace pg
