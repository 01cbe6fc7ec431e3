// The IEEE f64 step with each neighbour pair evaluated once (ARITH_F64_EXACT).
//
// The oracle's pair terms (oracle/prestige_oracle.hpp, sph_pair_loop) are, per particle i and
// neighbour j in walk order,
//   continuity  dr_i += m_j (w F),                  w = (v_i - v_j) . (x_i - x_j)
//   momentum    a_i  -= m_j (((P_i + P_j) + pi_ij) F) (x_i - x_j),
//               pi_ij = avk w / ((r^2 + eps h^2)(rho_i + rho_j)) where w < 0, else 0,
// with F, r^2 and w computed from the pair's differences.  In IEEE arithmetic every one of
// r^2, F, w, w F and X = ((P_i + P_j) + pi_ij) F is the same bit pattern from either side of
// the pair: negating both factors of a product is exact, the component sums run in the same
// order, and a + b == b + a.  Only m_j and the final difference vector belong to one side.  So
// the side with the lower slot evaluates the pair once and writes the symmetric value into both
// list entries; each particle then sums its own entries in list (walk) order, which is the
// oracle's order, bit for bit.
//
// Lists (sph_list_kernel) hold each slot's neighbours in ascending slot order: the entries below
// the slot's own index come first.  Per step:
//   sym_c1  for the entries above the slot (partner t > k): r^2, F, w, w F and r^2 + eps h^2 into
//           the slot's entry planes; the position of k in t's list (binary search: t's list is
//           ascending) into the mirror-index plane, and w F into t's entry there.
//   sym_c2  every entry in order: w F from the entry (own, or the mirror t wrote), times m_t,
//           into the continuity sum; then rho' and the packed {rho', P'} (the oracle's rho
//           update and Tait term).
//   sym_m1  for the entries above the slot: X from the stored F, w, r^2 + eps h^2 and the packed
//           {rho', P'} of both sides, into the slot's entry and through the mirror index.
//   sym_m2  every entry in order: X times m_t times the slot's own difference vector, into the
//           momentum sum; then the velocity and position update of fluid particles.
// A pair whose mirror entry does not exist (a list that reached its capacity before the partner:
// the partner's continued walk evaluates the pair itself) or was not written (the lower slot's
// list reached its capacity before this slot) is evaluated in full where it is read, and an
// overflowed list is followed by the rest of its candidate walk, evaluated in full, as in the
// other modes.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pg_arith.cuh"
#include "pg_internal.cuh"
#include "pg_kernels.cuh"
#include "pg_sph_pass.cuh"

namespace pg {
namespace {

using namespace sphpass;

typedef OpsD D;
constexpr uint32_t kNoMirror = 0xFFFFFFFFu;

// Entry planes of the per-entry store (a.fcache): doubles F, w, r^2 + eps h^2, S (w F after
// sym_c1, X after sym_m1), then the u32 mirror index, each plane in the tiled list layout.
struct Planes {
  double* base;
  size_t plane;  // entries per plane
  __device__ __forceinline__ double* F(size_t e) const { return base + e; }
  __device__ __forceinline__ double* W(size_t e) const { return base + plane + e; }
  __device__ __forceinline__ double* R(size_t e) const { return base + 2 * plane + e; }
  __device__ __forceinline__ double* S(size_t e) const { return base + 3 * plane + e; }
  __device__ __forceinline__ uint32_t* M(size_t e) const { return (uint32_t*)(base + 4 * plane) + e; }
};

__device__ __forceinline__ Planes planes_of(const SphArgs& a) {
  Planes p;
  p.base = (double*)a.fcache;
  p.plane = (size_t)((a.n + kListTile - 1) / kListTile) * kListTile * a.cap;
  return p;
}

__device__ __forceinline__ size_t entry(uint32_t k, uint32_t q, uint32_t cap) {
  return list_base(k, cap) + (size_t)q * kListTile;
}

// The oracle's pair geometry and continuity factor from slot k's side: d = x_k - x_t, r^2, F, w.
template <int DIM>
__device__ __forceinline__ void pair_geometry(const SphC<double>& c, const double4_32a& Ai, const double4_32a& Bi,
                                              const double4_32a& Aj, const double4_32a& Bj, double* d, double& r2,
                                              double& F, double& w) {
  d[0] = D::sub(Ai.x, Aj.x);
  d[1] = D::sub(Ai.y, Aj.y);
  d[2] = DIM == 3 ? D::sub(Ai.z, Aj.z) : 0.0;
  r2 = D::add(D::mul(d[0], d[0]), D::mul(d[1], d[1]));
  if (DIM == 3) r2 = D::add(r2, D::mul(d[2], d[2]));
  const double r = D::sqrt(r2);
  const double q = D::mul(r, c.inv_h);
  const double tq = D::sub(2.0, q);
  const double Fnear = D::mul(c.fa, D::sub(D::mul(2.25, q), 3.0));
  const double Ffar = D::div(D::mul(c.fb, D::mul(tq, tq)), r);
  F = q < 1.0 ? Fnear : Ffar;
  const double dv0 = D::sub(Bi.x, Bj.x), dv1 = D::sub(Bi.y, Bj.y);
  const double dv2 = DIM == 3 ? D::sub(Bi.z, Bj.z) : 0.0;
  w = D::add(D::mul(dv0, d[0]), D::mul(dv1, d[1]));
  if (DIM == 3) w = D::add(w, D::mul(dv2, d[2]));
}

// X = ((P_k + P_t) + pi_kt) F, the oracle's operation order.
__device__ __forceinline__ double momentum_factor(const SphC<double>& c, double F, double w, double r2e,
                                                  const double2& qk, const double2& qt) {
  const double av = D::div(D::mul(c.avk, w), D::mul(r2e, D::add(qk.x, qt.x)));
  const double pij = w < 0.0 ? av : 0.0;
  return D::mul(D::add(D::add(qk.y, qt.y), pij), F);
}

// The oracle's neighbour test on the candidate walk (r^2 < 4h^2 and r^2 > 0).
template <int DIM>
__device__ __forceinline__ bool is_neighbor(const SphC<double>& c, const double4_32a& Ai, const double4_32a& Aj) {
  const double d0 = D::sub(Ai.x, Aj.x), d1 = D::sub(Ai.y, Aj.y);
  double r2 = D::add(D::mul(d0, d0), D::mul(d1, d1));
  if (DIM == 3) {
    const double d2 = D::sub(Ai.z, Aj.z);
    r2 = D::add(r2, D::mul(d2, d2));
  }
  return r2 < c.four_h2 && r2 > 0.0;
}

// The rest of the candidate walk of slot k after its list reached capacity, in walk order
// (rows z, then y; slots ascending), calling on_pair(t) for every neighbour.
template <int DIM, class OnPair>
__device__ __forceinline__ void resume_walk(const SphArgs& a, const SphK& K, uint32_t k, const double4_32a& Ai,
                                            OnPair&& on_pair) {
  const float4* __restrict__ PF = (const float4*)a.s[3];
  const double4_32a* __restrict__ A = (const double4_32a*)a.s[0];
  const SphK* Kp;
  const Target T = target_of(a, k, &Kp, a.reach);
  const GridK& g = K.g;
  const int R = a.reach, RZ = DIM == 3 ? R : 0, side = 2 * R + 1, nrows = side * (2 * RZ + 1);
  const float4 pi = PF[k];
  const float thr = prefilter_threshold<false>(K, pi);
  const int row0 = (int)a.nresume[2 * (size_t)k];
  const uint32_t t0 = a.nresume[2 * (size_t)k + 1];
  for (int row = row0; row < nrows; ++row) {
    const int z = T.cz + row / side - RZ, y = T.cy + row % side - R;
    if (z < 0 || z >= g.nz || y < 0 || y >= g.ny) continue;
    const uint32_t rb = g.cell_base + ((uint32_t)z * g.ny + (uint32_t)y) * g.nx;
    const uint32_t e = a.cell_start[rb + T.x1 + 1];
    for (uint32_t t = row == row0 ? t0 : a.cell_start[rb + T.x0]; t < e; ++t)
      if (prefilter_hit<DIM, false>(pi, PF[t], thr) && is_neighbor<DIM>(K.d, Ai, A[t])) on_pair(t);
  }
}

// Slot t's list holds slot k (a neighbour above t) as a stored entry, so t wrote the pair's
// value into k's entry: t's list did not reach capacity before k (the list is ascending, so
// then its last stored entry is at least k).
__device__ __forceinline__ bool holds(const SphArgs& a, uint32_t t, uint32_t k) {
  if (a.nlen[t] <= a.cap) return true;
  return a.nlist[entry(t, a.cap - 1, a.cap)] >= k;
}

// First of the L entries of an ascending tiled list that is not below k.
__device__ __forceinline__ uint32_t lower_bound(const uint32_t* __restrict__ list, uint32_t L, uint32_t k) {
  uint32_t lo = 0, hi = L;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (list[(size_t)mid * kListTile] < k) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Position of k in slot t's stored list, or kNoMirror.
__device__ __forceinline__ uint32_t find_in_list(const SphArgs& a, uint32_t t, uint32_t k) {
  const uint32_t L = min(a.nlen[t], a.cap);
  const uint32_t* __restrict__ lt = a.nlist + list_base(t, a.cap);
  const uint32_t q = lower_bound(lt, L, k);
  return q < L && lt[(size_t)q * kListTile] == k ? q : kNoMirror;
}

struct Slot {
  uint32_t k, id, L;
  bool overflow;
};

__device__ __forceinline__ bool slot_of(const SphArgs& a, Slot& s) {
  s.k = a.k_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (s.k >= a.k_end) return false;
  s.id = a.sorted_id[s.k];
  const uint32_t cnt = a.nlen[s.k];
  s.L = min(cnt, a.cap);
  s.overflow = cnt > a.cap;
  return true;
}

// split > 0: the lists of the slots from split on may still be being built (on another stream).
// A slot's pair values need its partners' complete lists, so the first launch (second == 0)
// takes the slots below split whose stored partners all lie below split (lists ascend, so the
// last stored entry decides) and the second launch, after all lists, the others.
template <int DIM>
__global__ void __launch_bounds__(kSphMaxThreads) sym_c1_kernel(SphArgs a, uint32_t split, int second) {
  Slot s;
  if (!slot_of(a, s)) return;
  const uint32_t* __restrict__ my = a.nlist + list_base(s.k, a.cap);
  if (split) {
    const bool early = s.k < split && (s.L == 0 || my[(size_t)(s.L - 1) * kListTile] < split);
    if (early == (second != 0)) return;
  }
  const SphK& K = a.sys[sys_of_slot(a, s.id)];
  const double4_32a* __restrict__ A = (const double4_32a*)a.s[0];
  const double4_32a* __restrict__ B = (const double4_32a*)a.s[1];
  const Planes P = planes_of(a);
  const double4_32a Ai = A[s.k], Bi = B[s.k];
  // all lanes at the same entry index, so the entry-plane stores coalesce (starting each lane at
  // its own first upper entry, found by binary search, measured the same)
  for (uint32_t q = 0; q < s.L; ++q) {
    const uint32_t t = my[(size_t)q * kListTile];
    if (t < s.k) continue;
    double d[3], r2, F, w;
    pair_geometry<DIM>(K.d, Ai, Bi, A[t], B[t], d, r2, F, w);
    const double wF = D::mul(w, F);
    const size_t e = entry(s.k, q, a.cap);
    *P.F(e) = F;
    *P.W(e) = w;
    *P.R(e) = D::add(r2, K.d.eps_h2);
    *P.S(e) = wF;
    const uint32_t m = find_in_list(a, t, s.k);
    *P.M(e) = m;
    if (m != kNoMirror) *P.S(entry(t, m, a.cap)) = wF;
  }
}

template <int DIM>
__global__ void __launch_bounds__(kSphMaxThreads) sym_c2_kernel(SphArgs a) {
  Slot s;
  if (!slot_of(a, s)) return;
  const SphK& K = a.sys[sys_of_slot(a, s.id)];
  const SphC<double>& c = K.d;
  const double4_32a* __restrict__ A = (const double4_32a*)a.s[0];
  const double4_32a* __restrict__ B = (const double4_32a*)a.s[1];
  const Planes P = planes_of(a);
  const double4_32a Ai = A[s.k], Bi = B[s.k];
  const uint32_t* __restrict__ my = a.nlist + list_base(s.k, a.cap);
  auto full = [&](uint32_t t) {
    double d[3], r2, F, w;
    pair_geometry<DIM>(c, Ai, Bi, A[t], B[t], d, r2, F, w);
    return D::mul(w, F);
  };
  // software pipeline: list entries two ahead, the partner's mass and list length and the
  // entry's stored value one ahead (the pass waits on these loads; its FP64 work is two
  // operations per entry, summed in list order)
  double dr = 0.0;
  const uint32_t L = s.L;
  uint32_t t = L > 0 ? my[0] : 0u;
  uint32_t tn = L > 1 ? my[kListTile] : 0u;
  double mt = L > 0 ? A[t].w : 0.0;
  uint32_t nl = L > 0 ? a.nlen[t] : 0u;
  double sv = L > 0 ? *P.S(entry(s.k, 0, a.cap)) : 0.0;
  for (uint32_t q = 0; q < L; ++q) {
    const uint32_t tnn = q + 2 < L ? my[(size_t)(q + 2) * kListTile] : 0u;
    const double mtn = q + 1 < L ? A[tn].w : 0.0;
    const uint32_t nln = q + 1 < L ? a.nlen[tn] : 0u;
    const double svn = q + 1 < L ? *P.S(entry(s.k, q + 1, a.cap)) : 0.0;
    // the value is in the entry unless the partner below is one whose list did not reach this
    // slot (holds())
    const bool stored = t > s.k || nl <= a.cap || a.nlist[entry(t, a.cap - 1, a.cap)] >= s.k;
    dr = D::add(dr, D::mul(mt, stored ? sv : full(t)));
    t = tn;
    tn = tnn;
    mt = mtn;
    nl = nln;
    sv = svn;
  }
  if (s.overflow) resume_walk<DIM>(a, K, s.k, Ai, [&](uint32_t t) { dr = D::add(dr, D::mul(A[t].w, full(t))); });
  double* rho = (double*)a.rho;
  const double rn = D::add(rho[s.id], D::mul(c.dt, dr));
  rho[s.id] = rn;
  ((double2*)a.s[2])[s.k] = make_double2(rn, tait_pterm<D>(c, K.gamma, rn));
}

template <int DIM>
__global__ void __launch_bounds__(kSphMaxThreads) sym_m1_kernel(SphArgs a) {
  Slot s;
  if (!slot_of(a, s)) return;
  const SphK& K = a.sys[sys_of_slot(a, s.id)];
  const double2* __restrict__ Q = (const double2*)a.s[2];
  const Planes P = planes_of(a);
  const double2 qk = Q[s.k];
  const uint32_t* __restrict__ my = a.nlist + list_base(s.k, a.cap);
  // all lanes at the same entry index, so the loads of the entry planes coalesce (this pass does
  // little FP64 work per pair; starting each lane at its own first upper entry spread them over
  // the lines of different entry rows and the pass took 20 % longer)
  for (uint32_t q = 0; q < s.L; ++q) {
    const uint32_t t = my[(size_t)q * kListTile];
    if (t < s.k) continue;
    const size_t e = entry(s.k, q, a.cap);
    const double X = momentum_factor(K.d, *P.F(e), *P.W(e), *P.R(e), qk, Q[t]);
    *P.S(e) = X;
    const uint32_t m = *P.M(e);
    if (m != kNoMirror) *P.S(entry(t, m, a.cap)) = X;
  }
}

template <int DIM>
__global__ void __launch_bounds__(kSphMaxThreads) sym_m2_kernel(SphArgs a) {
  Slot s;
  if (!slot_of(a, s)) return;
  const SphK& K = a.sys[sys_of_slot(a, s.id)];
  const SphC<double>& c = K.d;
  const double4_32a* __restrict__ A = (const double4_32a*)a.s[0];
  const double4_32a* __restrict__ B = (const double4_32a*)a.s[1];
  const double2* __restrict__ Q = (const double2*)a.s[2];
  const Planes P = planes_of(a);
  const double4_32a Ai = A[s.k];
  const double2 qk = Q[s.k];
  const uint32_t* __restrict__ my = a.nlist + list_base(s.k, a.cap);
  double acc[3] = {0.0, 0.0, 0.0};
  // a pair without a stored X: everything from the packs
  auto full = [&](uint32_t t, const double4_32a& Aj) {
    double d[3], r2, F, w;
    pair_geometry<DIM>(c, Ai, B[s.k], Aj, B[t], d, r2, F, w);
    return momentum_factor(c, F, w, D::add(r2, c.eps_h2), qk, Q[t]);
  };
  auto add = [&](const double4_32a& Aj, double X) {
    const double coef = D::mul(Aj.w, X);
    acc[0] = D::sub(acc[0], D::mul(coef, D::sub(Ai.x, Aj.x)));
    acc[1] = D::sub(acc[1], D::mul(coef, D::sub(Ai.y, Aj.y)));
    if (DIM == 3) acc[2] = D::sub(acc[2], D::mul(coef, D::sub(Ai.z, Aj.z)));
  };
  for (uint32_t q = 0; q < s.L; ++q) {
    const uint32_t t = my[(size_t)q * kListTile];
    const double4_32a Aj = A[t];
    add(Aj, t > s.k || holds(a, t, s.k) ? *P.S(entry(s.k, q, a.cap)) : full(t, Aj));
  }
  if (s.overflow) resume_walk<DIM>(a, K, s.k, Ai, [&](uint32_t t) {
      const double4_32a Aj = A[t];
      add(Aj, full(t, Aj));
    });
  if (s.id < K.fluid_end) {
    double* pos = (double*)a.pos;
    double* vel = (double*)a.vel;
#pragma unroll
    for (int cc = 0; cc < DIM; ++cc) {
      const size_t o = (size_t)s.id * DIM + cc;
      const double v = D::add(vel[o], D::mul(c.dt, D::add(acc[cc], c.g[cc])));
      vel[o] = v;
      pos[o] = D::add(pos[o], D::mul(c.dt, v));
    }
  }
}

typedef void (*SymKernel)(SphArgs);

template <int DIM>
SymKernel sym_kernel(int part) {
  switch (part) {
    case 1: return sym_c2_kernel<DIM>;
    case 2: return sym_m1_kernel<DIM>;
    case 3: return sym_m2_kernel<DIM>;
    default: return nullptr;
  }
}

}  // namespace

size_t sph_sym_entry_bytes() { return 4 * sizeof(double) + sizeof(uint32_t); }

int launch_sph_sym(cudaStream_t st, const SphArgs& a, int part, int block, uint32_t split, int second) {
  SymKernel kern = a.dim == 2 ? sym_kernel<2>(part) : sym_kernel<3>(part);
  if (!kern && part != 0) {
    set_error("unknown part %d of the pair-once step", part);
    return PG_EINVAL;
  }
  if (block < 32 || block > kSphMaxThreads || block % 32) {
    set_error("block size %d must be a multiple of 32 in 32..%d", block, kSphMaxThreads);
    return PG_EINVAL;
  }
  if (a.k_end <= a.k_begin) return PG_OK;
  const unsigned blocks = (unsigned)((a.k_end - a.k_begin + block - 1) / block);
  if (part == 0) {
    if (a.dim == 2) sym_c1_kernel<2><<<blocks, block, 0, st>>>(a, split, second);
    else sym_c1_kernel<3><<<blocks, block, 0, st>>>(a, split, second);
  } else {
    kern<<<blocks, block, 0, st>>>(a);
  }
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

}  // namespace pg
