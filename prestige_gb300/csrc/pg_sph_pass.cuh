// The SPH pair-pass skeleton shared by the forward passes (pg_sph.cu) and the adjoint passes
// (pg_adjoint.cu): the candidate walk over the neighbour rows with its FP32 prefilter, the
// neighbour-list kernel built on it, the list-driven pair pass (one thread per target slot) and
// the Tait pressure term.
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
  T.live = k0 < a.k_end;
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

// FP32 r^2 below which |x_j - x_i| < 2h holds in f64 for certain: the mirror image of
// prefilter_threshold (same error bound delta, taken off instead of added).
__device__ __forceinline__ float certain_threshold(const SphK& K, const float4& pi) {
  const float M = fmaxf(fmaxf(fabsf(pi.x), fabsf(pi.y)), fabsf(pi.z)) + K.two_h_f;
  const float delta = 2.384185791015625e-07f * (2.f * M + K.two_h_f);
  const float rr = fmaxf(K.two_h_f - 2.f * delta, 0.f);
  return rr * rr * 0.9999847f;
}

// The oracle's f64 neighbour test of slots k and t (positions X, double4 per slot); inline in
// the list kernel, called out of line by the pair passes (exact_neighbor_call), where the f64
// registers would otherwise count against the pair loop.
template <int DIM>
__device__ __forceinline__ bool exact_neighbor(const double4_32a* X, uint32_t k, uint32_t t, double four_h2) {
  const double4_32a xi = X[k], xj = X[t];
  const double d0 = __dsub_rn(xi.x, xj.x), d1 = __dsub_rn(xi.y, xj.y);
  double r2 = __dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1));
  if (DIM == 3) {
    const double d2 = __dsub_rn(xi.z, xj.z);
    r2 = __dadd_rn(r2, __dmul_rn(d2, d2));
  }
  return r2 < four_h2 && r2 > 0.0;
}

template <int DIM>
__device__ __noinline__ bool exact_neighbor_call(const double4_32a* X, uint32_t k, uint32_t t, double four_h2) {
  return exact_neighbor<DIM>(X, k, t, four_h2);
}

// FP32 r^2 of a candidate, in the operation order of the prefilter (EXACT_PF: IEEE single, no
// contraction; otherwise with fused multiply-add).
template <int DIM, bool EXACT_PF>
__device__ __forceinline__ float candidate_r2(const float4& pi, const float4& pj) {
  if (EXACT_PF) {
    const float d0 = __fsub_rn(pi.x, pj.x), d1 = __fsub_rn(pi.y, pj.y);
    float r2 = __fadd_rn(__fmul_rn(d0, d0), __fmul_rn(d1, d1));
    if (DIM == 3) {
      const float d2 = __fsub_rn(pi.z, pj.z);
      r2 = __fadd_rn(r2, __fmul_rn(d2, d2));
    }
    return r2;
  }
  const float d0 = pi.x - pj.x, d1 = pi.y - pj.y;
  float r2 = fmaf(d1, d1, d0 * d0);
  if (DIM == 3) {
    const float d2 = pi.z - pj.z;
    r2 = fmaf(d2, d2, r2);
  }
  return r2;
}

// List membership of a candidate for target k (t != k is tested by the caller).  XD < 0: the FP32
// prefilter (hit; a superset of the neighbours, the pair passes repeat the exact test).
// XD >= 0: exactly the oracle's f64 test.  hit: a neighbour for certain; below: under the
// conservative threshold.  Candidates below but not hit (a narrow band around (2h)^2, and
// coincident FP32 positions) are left to exact_neighbor on the f64 positions a.s[XD].
template <int DIM, bool EXACT_PF, int XD>
__device__ __forceinline__ void classify(const float4& pi, const float4& pj, float thr, float thr_lo, bool& hit,
                                         bool& below) {
  const float r2 = candidate_r2<DIM, EXACT_PF>(pi, pj);
  if (XD < 0) {
    hit = r2 < thr && (!EXACT_PF || r2 > 0.f);
    below = false;
  } else {
    hit = r2 < thr_lo && r2 > 0.f;
    below = r2 < thr;
  }
}

// ---------------------------------------------------------------------------------------
// Neighbour lists.  sph_list_kernel walks the candidates of every slot once per step and writes
// the listed slots (classify: with XD < 0 the FP32 test (exact for f32 systems), with XD >= 0
// exactly the f64 neighbours;
// never the slot itself) in walk order (rows z, then y ascending; slots ascending along a row)
// to nlist in warp tiles (list_base: entry q of the 32 slots of a tile is one 128-byte line, so a
// warp's reads of one entry index coalesce and its writes fill whole sectors while they are in
// L2); nlen[k] = number of listed slots (may exceed cap).  When the list fills, nresume[2k],
// [2k+1] = (row, slot) of the first listed candidate that did not fit, so the pair passes can
// continue the walk from there.
//
// Each lane walks its own rows, kListBatch candidates at a time: loads without a clamp (the
// packs are padded by kPackPad records), the FP32 classification folded into bit masks, the rare
// f64 band tests once per batch, then the pushes of the batch's hits in order.  The next row's
// slot range is loaded while the current row is walked.  Lanes whose targets share a cell walk
// the same candidates in step, so their loads coalesce (pruning each lane's rows to the cells
// its own target can reach was measured: it breaks that, and the walk got slower).
// ---------------------------------------------------------------------------------------
constexpr int kListBatch = 16;
static_assert(kPackPad >= (size_t)kListBatch - 1, "sorted packs must be padded for a whole batch past the end");

// Offset of slot k's entry 0 in the tiled list array (entry q at + q * kListTile).
__device__ __forceinline__ size_t list_base(uint32_t k, uint32_t cap) {
  return (size_t)(k / kListTile) * cap * kListTile + (k % kListTile);
}

__device__ __forceinline__ void list_push(const SphArgs& a, uint32_t* my, uint32_t& cnt, uint32_t k, int row,
                                          uint32_t t) {
  if (cnt < a.cap) {
    my[(size_t)cnt * kListTile] = t;
  } else if (cnt == a.cap) {
    a.nresume[2 * (size_t)k] = (uint32_t)row;
    a.nresume[2 * (size_t)k + 1] = t;
  }
  ++cnt;
}

template <int DIM, bool EXACT_PF, int XD>
__global__ void __launch_bounds__(kSphMaxThreads) sph_list_kernel(SphArgs a, int pf_index) {
  const int tid = threadIdx.x;
  const float4* __restrict__ PF = (const float4*)a.s[pf_index];
  const double4_32a* __restrict__ X = (const double4_32a*)a.s[XD < 0 ? 0 : XD];
  const uint32_t* __restrict__ start = a.cell_start;
  const int R = a.reach;
  const int RZ = DIM == 3 ? R : 0;
  const int side = 2 * R + 1;
  const int nrows = side * (2 * RZ + 1);
  const uint32_t bs = blockDim.x;
  const uint32_t tile1 = (a.k_end + bs - 1) / bs;

  for (uint32_t tile = a.k_begin / bs + blockIdx.x; tile < tile1; tile += gridDim.x) {
    const SphK* Kp;
    const Target T = target_of(a, tile * bs + tid, &Kp, R);
    const SphK& K = *Kp;
    const GridK& g = K.g;
    const float4 pi = PF[T.k];
    const float thr = prefilter_threshold<EXACT_PF>(K, pi);
    const float thr_lo = XD < 0 ? 0.f : certain_threshold(K, pi);
    uint32_t* __restrict__ my = a.nlist + list_base(T.k, a.cap);  // entry q at my[q * kListTile]
    uint32_t cnt = 0;
    // slot range of a row (empty outside the grid); the next row's range is loaded while the
    // current row is walked
    auto row_range = [&](int r, uint32_t& a, uint32_t& b) {
      const int z = T.cz + r / side - RZ, y = T.cy + r % side - R;
      a = b = 0;
      if (T.live && z >= 0 && z < g.nz && y >= 0 && y < g.ny) {
        const uint32_t rb = g.cell_base + ((uint32_t)z * g.ny + (uint32_t)y) * g.nx;
        a = start[rb + T.x0];
        b = start[rb + T.x1 + 1];
      }
    };
    int row = -1, nxt = 0;
    uint32_t t = 0, e = 0, tn, en;
    row_range(0, tn, en);
    while (true) {
      while (t >= e && nxt < nrows) {
        t = tn;
        e = en;
        row = nxt++;
        if (nxt < nrows) row_range(nxt, tn, en);
      }
      if (t >= e) break;
      // the batch's candidates that belong to the row, the target itself left out (the packs
      // are padded by kPackPad records, so the loads need no clamp)
      unsigned valid = e - t >= (uint32_t)kListBatch ? (1u << kListBatch) - 1 : (1u << (e - t)) - 1;
      if (T.k - t < (uint32_t)kListBatch) valid &= ~(1u << (T.k - t));
      const float4* __restrict__ pb = PF + t;
      float4 pj[kListBatch];
#pragma unroll
      for (int b = 0; b < kListBatch; ++b) pj[b] = __ldg(pb + b);
      unsigned hit = 0, below = 0;
#pragma unroll
      for (int b = 0; b < kListBatch; ++b) {
        bool h, m;
        classify<DIM, EXACT_PF, XD>(pi, pj[b], thr, thr_lo, h, m);
        if (h) hit |= 1u << b;
        if (m) below |= 1u << b;
      }
      hit &= valid;
      if (XD >= 0) {
        for (unsigned m = below & ~hit & valid; m; m &= m - 1) {
          const int b = __ffs(m) - 1;
          if (exact_neighbor<DIM>(X, T.k, t + b, K.d.four_h2)) hit |= 1u << b;
        }
      }
      for (; hit; hit &= hit - 1) list_push(a, my, cnt, T.k, row, t + __ffs(hit) - 1);
      t += kListBatch;
    }
    if (T.live) a.nlen[T.k] = cnt;
  }
}

// L2 prefetch hint for one address (PTX prefetch.global.L2; a hint, it returns nothing).
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// List entries (and, for policies with kL2Entry, the policy's own per-entry data through
// prefetch_entry(q)) are prefetched into L2 this many entries ahead of their use: both are
// streams from DRAM, read once, that the one-entry-ahead register prefetch cannot cover.
constexpr uint32_t kL2Ahead = 8;

template <class P, class = void>
struct L2EntryPolicy {
  static constexpr bool value = false;
};
template <class P>
struct L2EntryPolicy<P, decltype((void)P::kL2Entry)> {
  static constexpr bool value = P::kL2Entry;
};

// Policies that split a pair into fetch(t, q) (the loads for neighbour t, entry q of the list) and
// pair_with(t, q, fetched).
template <class P, class = void>
struct PrefetchPolicy {
  static constexpr bool value = false;
};
template <class P>
struct PrefetchPolicy<P, decltype((void)P::kPrefetch)> {
  static constexpr bool value = P::kPrefetch;
};

// Pair pass over the lists of sph_list_kernel (any block size up to kSphMaxThreads, a
// multiple of 32).  LANES consecutive threads share one target slot (32 / LANES particles per
// warp): lane `sub` of a slot takes its list entries sub, sub + LANES, ..., the lanes' partial
// sums are combined by the policy's reduce_lanes<LANES>() (a fixed butterfly, so the result is
// deterministic) and lane 0 writes the slot's results.  LANES > 1 changes the summation order,
// so only the tolerance-based modes (double-word f64, contracted f32) use it.  Lanes step
// through their lists together; a list that overflowed is followed by the rest of the walk from
// its resume point (lane 0).
template <class Pairs, int DIM, bool EXACT_PF, int LANES = 1>
__global__ void __launch_bounds__(kSphMaxThreads) sph_list_pass_kernel(SphArgs a, int pf_index) {
  static_assert(LANES == 1 || LANES == 2 || LANES == 4, "1, 2 or 4 lanes per slot");
  const int tid = threadIdx.x;
  const uint32_t cap = a.cap;
  const uint32_t spb = blockDim.x / LANES;  // slots per block
  const uint32_t sub = LANES > 1 ? (uint32_t)tid % LANES : 0u;
  const uint32_t tile1 = (a.k_end + spb - 1) / spb;
  for (uint32_t tile = a.k_begin / spb + blockIdx.x; tile < tile1; tile += gridDim.x) {
    const uint32_t k0 = tile * spb + (uint32_t)tid / LANES;
    const bool live = k0 < a.k_end;
    const uint32_t k = live ? k0 : a.n - 1;
    const uint32_t id = a.sorted_id[k];
    const SphK& K = a.sys[sys_of_slot(a, id)];
    Pairs P;
    P.begin(a, K, k);
    const uint32_t cnt = live ? a.nlen[k] : 0u;
    const uint32_t L = min(cnt, cap);
    const uint32_t* __restrict__ my = a.nlist + list_base(k, cap);  // entry q at my[q * kListTile]
    if constexpr (PrefetchPolicy<Pairs>::value) {
      // software pipeline: list entries two ahead, the neighbour's pack records one ahead; the
      // unrolled pair bodies (branch-free) interleave
      constexpr uint32_t S = LANES;
      const uint32_t q0 = sub;
      uint32_t t = q0 < L ? my[q0 * kListTile] : k;
      uint32_t tn = q0 + S < L ? my[(q0 + S) * kListTile] : t;
      typename Pairs::Pre cur = P.fetch(t, q0 < L ? q0 : 0);
#pragma unroll 2
      for (uint32_t q = q0; q < L; q += S) {
        if (q + kL2Ahead * S < L) {
          prefetch_l2(my + (size_t)(q + kL2Ahead * S) * kListTile);
          if constexpr (L2EntryPolicy<Pairs>::value) P.prefetch_entry(q + kL2Ahead * S);
        }
        const uint32_t tnn = q + 2 * S < L ? my[(q + 2 * S) * kListTile] : tn;
        const typename Pairs::Pre nxt = P.fetch(tn, q + S < L ? q + S : q);
        P.pair_with(t, q, cur);
        cur = nxt;
        t = tn;
        tn = tnn;
      }
    } else {
      for (uint32_t q = sub; q < L; q += LANES) P.pair(my[q * kListTile]);
    }
    if (cnt > cap && sub == 0) {
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
    if constexpr (LANES > 1) P.template reduce_lanes<LANES>();  // whole warps: the tile loop is uniform
    if (live && sub == 0) P.finish(a, K, id, k);
  }
}

}  // namespace sphpass
}  // namespace pg
