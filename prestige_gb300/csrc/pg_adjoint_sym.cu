// The FP64 adjoint passes with each neighbour pair evaluated once (IEEE f64 handles).
//
// The adjoint of one step (pg_adjoint.cu) sums, for particle i over its neighbours j, the
// derivatives of the pair terms Lam_M and Lam_C.  With x = x_i - x_j, v = v_i - v_j and
// E = m_j abar_i - m_i abar_j, particle i's share of a pair is
//   momentum     gx_i += a1 x + b1 v - F S E,   gv_i += b1 x,   gr_i -= F (x.E) (P'_i - Pi / rho_ij)
//   continuity   gx_i += G w D x + F D v,       gv_i += F D x
// where a1, b1, F, G, S, Pi, w, x.E and D are the same from either side of the pair while x, v
// and E change sign.  So j's share is the negated vector of i's (and its own P'_j in gr), and
// the lower slot of a pair evaluates it once:
//   adj_mirror  for each entry above the slot, the slot's position in the partner's list
//           (binary search: the partner's list is ascending), or none.
//   adj_a1  (entries above the slot) the momentum terms; its own share into per-slot partial
//           sums; the partner's share (the vectors, F x.E and Pi / rho_ij) into the partner's list
//           entry at the mirror index; the pair's continuity vectors U1 = G w x + F v and
//           U2 = F x and the partner's mass into the slot's own entry; the parameter derivatives
//           of the pair whole (half of each when the partner evaluates its side itself).
//   adj_a2  (entries below the slot, in list order) the partners' shares, then the momentum
//           update of lx, lv, lr, the parameter sums and dbar = dt lr for the continuity pass.
//   adj_c1 / adj_c2  the same for the continuity terms: the slot's share is D U1 and D U2 with
//           D = dbar_k m_t + dbar_t m_k (dbar from adj_a2), the partner's the negated vectors.
// A pair that is not held by both lists (a list that reached its capacity) is evaluated by each
// side for itself, as in the two-sided passes, with half of the parameter derivatives each; the
// rest of an overflowed list's walk likewise.  The sums run in a different order from the
// two-sided passes, within the adjoint's tolerance against the dual-number oracle.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pg_arith.cuh"
#include "pg_internal.cuh"
#include "pg_kernels.cuh"
#include "pg_sph_pass.cuh"

namespace pg {
namespace {

using namespace sphpass;

constexpr uint32_t kNoMirror = 0xFFFFFFFFu;
constexpr int kPlanes = 15;  // doubles per list entry (plus one u32)
// the partner's momentum share (Vx, Vv, F x.E, Pi / rho_ij); for the continuity pass, the pair's
// vectors U1 = G w x + F v and U2 = F x and the partner's mass (own entries above the slot)
enum { kMx = 0, kMv = 3, kFxE = 6, kPIrb = 7, kU1 = 8, kU2 = 11, kMt = 14 };
constexpr int kSlotSums = 9;  // per-slot partial sums: gx (3), gv (3), gr, gal, gB

struct Planes {
  double* base;
  size_t plane;  // entries per plane
  __device__ __forceinline__ double& at(int j, size_t e) const { return base[j * plane + e]; }
  __device__ __forceinline__ uint32_t& mirror(size_t e) const { return ((uint32_t*)(base + kPlanes * plane))[e]; }
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

// Slot t's list holds slot k (a neighbour above t) as a stored entry.
__device__ __forceinline__ bool holds(const SphArgs& a, uint32_t t, uint32_t k) {
  if (a.nlen[t] <= a.cap) return true;
  return a.nlist[entry(t, a.cap - 1, a.cap)] >= k;
}

// Position of k in slot t's stored (ascending) list, or kNoMirror.
__device__ __forceinline__ uint32_t find_in_list(const SphArgs& a, uint32_t t, uint32_t k) {
  const uint32_t L = min(a.nlen[t], a.cap);
  const uint32_t* __restrict__ lt = a.nlist + list_base(t, a.cap);
  uint32_t lo = 0, hi = L;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (lt[(size_t)mid * kListTile] < k) lo = mid + 1;
    else hi = mid;
  }
  return lo < L && lt[(size_t)lo * kListTile] == k ? lo : kNoMirror;
}

// Index of the first entry above slot k in its ascending list of L entries (binary search):
// the entries before it are the ones below k.
__device__ __forceinline__ uint32_t first_above(const uint32_t* __restrict__ my, uint32_t L, uint32_t k) {
  uint32_t lo = 0, hi = L;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (my[(size_t)mid * kListTile] < k) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// The slot-ordered packs of the adjoint step (adjoint_prep_kernel):
//   s0 X {x, y, z, m}  s1 V {v, rho'}  s2 Q {P, P', P/B}  s3 A {abar}  s4 float4 x  s5 dbar
//   s6 per-slot partial sums (kSlotSums planes of n doubles)
struct Packs {
  const double4_32a *X, *V, *Q, *A;
  const double* DB;
  double* PS;
  __device__ __forceinline__ Packs(const SphArgs& a)
      : X((const double4_32a*)a.s[0]), V((const double4_32a*)a.s[1]), Q((const double4_32a*)a.s[2]),
        A((const double4_32a*)a.s[3]), DB((const double*)a.s[5]), PS((double*)a.s[6]) {}
};

// Pair geometry from slot k's side: x, v, r^2, F = (dW/dr)/r, G = (dF/dr)/r, w = v . x.
template <int DIM>
struct Geo {
  double d[3], dv[3], r2, F, G, w;
};

template <int DIM>
__device__ __forceinline__ Geo<DIM> geometry(const SphC<double>& c, const double4_32a& xk, const double4_32a& vk,
                                             const double4_32a& xt, const double4_32a& vt) {
  Geo<DIM> g;
  g.d[0] = xk.x - xt.x;
  g.d[1] = xk.y - xt.y;
  g.d[2] = DIM == 3 ? xk.z - xt.z : 0.0;
  g.r2 = __dadd_rn(__dmul_rn(g.d[0], g.d[0]), __dmul_rn(g.d[1], g.d[1]));
  if (DIM == 3) g.r2 = __dadd_rn(g.r2, __dmul_rn(g.d[2], g.d[2]));
  const double inv_r = rsqrt(g.r2);  // one FP64 sequence in place of a square root and a division
  const double r = g.r2 * inv_r;
  const double q = r * c.inv_h;
  if (q < 1.0) {
    g.F = c.fa * (2.25 * q - 3.0);
    g.G = c.fa * 2.25 * c.inv_h * inv_r;
  } else {
    const double tq = 2.0 - q;
    g.F = c.fb * tq * tq * inv_r;
    g.G = -(c.fb * tq * inv_r) * (2.0 * c.inv_h + tq * inv_r) * inv_r;
  }
  g.dv[0] = vk.x - vt.x;
  g.dv[1] = vk.y - vt.y;
  g.dv[2] = DIM == 3 ? vk.z - vt.z : 0.0;
  g.w = g.dv[0] * g.d[0] + g.dv[1] * g.d[1];
  if (DIM == 3) g.w += g.dv[2] * g.d[2];
  return g;
}

// The oracle's neighbour test (r^2 < 4h^2 and r^2 > 0), for the continued walks.
template <int DIM>
__device__ __forceinline__ bool is_neighbor(const SphC<double>& c, const double4_32a& xk, const double4_32a& xt) {
  const double d0 = xk.x - xt.x, d1 = xk.y - xt.y;
  double r2 = __dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1));
  if (DIM == 3) {
    const double d2 = xk.z - xt.z;
    r2 = __dadd_rn(r2, __dmul_rn(d2, d2));
  }
  return r2 < c.four_h2 && r2 > 0.0;
}

// The momentum-adjoint terms of pair (k, t) from k's side.
template <int DIM>
struct MomTerms {
  double Vx[3], Vv[3], FxE, PIrb, gal, gB;  // gal, gB: the whole pair's parameter derivatives
  double U1[3], U2[3], mt;                  // the continuity share is D U1, D U2
};

template <int DIM>
__device__ __forceinline__ MomTerms<DIM> mom_terms(const SphK& K, const Packs& P, uint32_t k, uint32_t t,
                                                   const double4_32a& xk, const double4_32a& vk) {
  const SphC<double>& c = K.d;
  const double4_32a xt = P.X[t], vt = P.V[t], qk = P.Q[k], qt = P.Q[t], ak = P.A[k], at = P.A[t];
  const Geo<DIM> g = geometry<DIM>(c, xk, vk, xt, vt);
  const double mk = xk.w, mt = xt.w;
  const double rb = vk.w + vt.w;
  const double e = g.r2 + c.eps_h2;
  // one reciprocal serves the four quotients of the terms
  const double inv_erb = __drcp_rn(e * rb);
  const double inv_e = rb * inv_erb, inv_rb = e * inv_erb;
  double c1 = 0.0, c1a = 0.0;
  if (g.w < 0.0) {
    const double base = inv_e * inv_rb;
    c1 = c.avk * base;
    c1a = K.avk_alpha * base;
  }
  const double PI = c1 * g.w;
  const double S = qk.x + qt.x + PI;
  const double E[3] = {mt * ak.x - mk * at.x, mt * ak.y - mk * at.y, DIM == 3 ? mt * ak.z - mk * at.z : 0.0};
  double xE = 0.0;
#pragma unroll
  for (int cc = 0; cc < DIM; ++cc) xE += g.d[cc] * E[cc];
  const double a1 = -g.G * S * xE + 2.0 * g.F * xE * PI * inv_e;
  const double b1 = -g.F * c1 * xE;
  const double fs = g.F * S;
  MomTerms<DIM> m;
#pragma unroll
  for (int cc = 0; cc < 3; ++cc) {
    m.Vx[cc] = cc < DIM ? a1 * g.d[cc] + b1 * g.dv[cc] - fs * E[cc] : 0.0;
    m.Vv[cc] = cc < DIM ? b1 * g.d[cc] : 0.0;
  }
  m.FxE = g.F * xE;
  m.PIrb = PI * inv_rb;
  m.gal = m.FxE * c1a * g.w;
  m.gB = m.FxE * (qk.z + qt.z);
  const double GW = g.G * g.w;
#pragma unroll
  for (int cc = 0; cc < 3; ++cc) {
    m.U1[cc] = cc < DIM ? GW * g.d[cc] + g.F * g.dv[cc] : 0.0;
    m.U2[cc] = cc < DIM ? g.F * g.d[cc] : 0.0;
  }
  m.mt = mt;
  return m;
}

struct Sums {
  double gx[3], gv[3], gr, gal, gB;
};

template <int DIM>
__device__ __forceinline__ void add_own(Sums& s, const MomTerms<DIM>& m, double Pdk, double share) {
#pragma unroll
  for (int cc = 0; cc < DIM; ++cc) {
    s.gx[cc] += m.Vx[cc];
    s.gv[cc] += m.Vv[cc];
  }
  s.gr -= m.FxE * (Pdk - m.PIrb);
  s.gal -= share * m.gal;
  s.gB -= share * m.gB;
}

// The rest of the candidate walk of slot k after its list reached capacity (walk order).
template <int DIM, class OnPair>
__device__ __forceinline__ void resume_walk(const SphArgs& a, const SphK& K, const Packs& P, uint32_t k,
                                            const double4_32a& xk, OnPair&& on_pair) {
  const float4* __restrict__ PF = (const float4*)a.s[4];
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
      if (prefilter_hit<DIM, false>(pi, PF[t], thr) && is_neighbor<DIM>(K.d, xk, P.X[t])) on_pair(t);
  }
}

struct Slot {
  uint32_t k, id, L;
  bool overflow;
};

__device__ __forceinline__ bool slot_of(const SphArgs& a, Slot& s) {
  s.k = blockIdx.x * blockDim.x + threadIdx.x;
  if (s.k >= a.n) return false;
  s.id = a.sorted_id[s.k];
  const uint32_t cnt = a.nlen[s.k];
  s.L = min(cnt, a.cap);
  s.overflow = cnt > a.cap;
  return true;
}

__device__ __forceinline__ void store_sums(const SphArgs& a, const Packs& P, uint32_t k, const Sums& s, int count) {
  const double v[kSlotSums] = {s.gx[0], s.gx[1], s.gx[2], s.gv[0], s.gv[1], s.gv[2], s.gr, s.gal, s.gB};
  for (int j = 0; j < count; ++j) P.PS[(size_t)j * a.n + k] = v[j];
}

__device__ __forceinline__ Sums load_sums(const SphArgs& a, const Packs& P, uint32_t k, int count) {
  double v[kSlotSums] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int j = 0; j < count; ++j) v[j] = P.PS[(size_t)j * a.n + k];
  Sums s;
  for (int c = 0; c < 3; ++c) {
    s.gx[c] = v[c];
    s.gv[c] = v[3 + c];
  }
  s.gr = v[6];
  s.gal = v[7];
  s.gB = v[8];
  return s;
}

// The mirror index of every entry above its slot: the position of the slot in the partner's
// list (a binary search, latency-bound; apart from the FP64 work of adj_a1 it runs at full
// occupancy).
__global__ void __launch_bounds__(kSphMaxThreads) adj_mirror_kernel(SphArgs a) {
  Slot s;
  if (!slot_of(a, s)) return;
  const Planes E = planes_of(a);
  const uint32_t* __restrict__ my = a.nlist + list_base(s.k, a.cap);
  for (uint32_t q = 0; q < s.L; ++q) {
    const uint32_t t = my[(size_t)q * kListTile];
    if (t > s.k) E.mirror(entry(s.k, q, a.cap)) = find_in_list(a, t, s.k);
  }
}

template <int DIM>
__global__ void __launch_bounds__(kSphMaxThreads) adj_a1_kernel(SphArgs a) {
  Slot s;
  if (!slot_of(a, s)) return;
  const SphK& K = a.sys[0];
  const Packs P(a);
  const Planes E = planes_of(a);
  const double4_32a xk = P.X[s.k], vk = P.V[s.k];
  const double Pdk = P.Q[s.k].y;
  const uint32_t* __restrict__ my = a.nlist + list_base(s.k, a.cap);
  Sums sum = {{0, 0, 0}, {0, 0, 0}, 0, 0, 0};
  // each lane from its own first entry above the slot, so the lanes of a warp evaluate their
  // pairs in the same iterations
  for (uint32_t q = first_above(my, s.L, s.k); q < s.L; ++q) {
    const uint32_t t = my[(size_t)q * kListTile];
    const MomTerms<DIM> m = mom_terms<DIM>(K, P, s.k, t, xk, vk);
    const size_t e = entry(s.k, q, a.cap);
#pragma unroll
    for (int cc = 0; cc < DIM; ++cc) {
      E.at(kU1 + cc, e) = m.U1[cc];
      E.at(kU2 + cc, e) = m.U2[cc];
    }
    E.at(kMt, e) = m.mt;
    const uint32_t mt = E.mirror(e);
    if (mt != kNoMirror) {
      const size_t f = entry(t, mt, a.cap);
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) {
        E.at(kMx + cc, f) = m.Vx[cc];
        E.at(kMv + cc, f) = m.Vv[cc];
      }
      E.at(kFxE, f) = m.FxE;
      E.at(kPIrb, f) = m.PIrb;
    }
    add_own<DIM>(sum, m, Pdk, mt != kNoMirror ? 1.0 : 0.5);
  }
  store_sums(a, P, s.k, sum, kSlotSums);
}

template <int DIM>
__global__ void __launch_bounds__(kSphMaxThreads) adj_a2_kernel(SphArgs a) {
  Slot s;
  if (!slot_of(a, s)) return;
  const SphK& K = a.sys[0];
  const Packs P(a);
  const Planes E = planes_of(a);
  const double4_32a xk = P.X[s.k], vk = P.V[s.k];
  const double Pdk = P.Q[s.k].y;
  const uint32_t* __restrict__ my = a.nlist + list_base(s.k, a.cap);
  Sums sum = load_sums(a, P, s.k, kSlotSums);
  const uint32_t below = first_above(my, s.L, s.k);  // the entries below the slot come first
  for (uint32_t q = 0; q < below; ++q) {
    const uint32_t t = my[(size_t)q * kListTile];
    if (holds(a, t, s.k)) {  // t's share of the pair was written here by t: negate it
      const size_t e = entry(s.k, q, a.cap);
#pragma unroll
      for (int cc = 0; cc < DIM; ++cc) {
        sum.gx[cc] -= E.at(kMx + cc, e);
        sum.gv[cc] -= E.at(kMv + cc, e);
      }
      sum.gr -= E.at(kFxE, e) * (Pdk - E.at(kPIrb, e));
    } else {
      add_own<DIM>(sum, mom_terms<DIM>(K, P, s.k, t, xk, vk), Pdk, 0.5);
    }
  }
  if (s.overflow)
    resume_walk<DIM>(a, K, P, s.k, xk,
                     [&](uint32_t t) { add_own<DIM>(sum, mom_terms<DIM>(K, P, s.k, t, xk, vk), Pdk, 0.5); });
  // the momentum adjoint's update: lx += gx, lv += dt lx' (fluid) + gv, lr += gr, dbar = dt lr for
  // the continuity pass, and the parameter sums
  double* lx = (double*)a.lam[0];
  double* lv = (double*)a.lam[1];
  double* lr = (double*)a.lam[2];
  const bool fluid = s.id < K.fluid_end;
  const double dt = K.d.dt;
#pragma unroll
  for (int cc = 0; cc < DIM; ++cc) {
    const size_t o = (size_t)s.id * DIM + cc;
    const double lxo = lx[o];
    lx[o] = lxo + sum.gx[cc];
    lv[o] = (fluid ? lv[o] + dt * lxo : lv[o]) + sum.gv[cc];
  }
  const double lrt = lr[s.id] + sum.gr;
  lr[s.id] = lrt;
  ((double*)a.s[5])[s.k] = dt * lrt;
  ((double*)a.lam[3])[s.id] += sum.gal;
  ((double*)a.lam[4])[s.id] += sum.gB;
}

// The continuity-adjoint share of a pair from the slot's side is D U1 and D U2, with
// D = dbar_k m_t + dbar_t m_k, U1 = G w x + F v and U2 = F x.
template <int DIM>
__device__ __forceinline__ void cont_full(const SphK& K, const Packs& P, uint32_t k, uint32_t t, const double4_32a& xk,
                                          const double4_32a& vk, Sums& sum) {
  const double4_32a xt = P.X[t];
  const Geo<DIM> g = geometry<DIM>(K.d, xk, vk, xt, P.V[t]);
  const double D = P.DB[k] * xt.w + P.DB[t] * xk.w;
  const double GW = g.G * g.w;
#pragma unroll
  for (int cc = 0; cc < DIM; ++cc) {
    sum.gx[cc] += D * (GW * g.d[cc] + g.F * g.dv[cc]);
    sum.gv[cc] += D * (g.F * g.d[cc]);
  }
}

template <int DIM>
__global__ void __launch_bounds__(kSphMaxThreads) adj_c1_kernel(SphArgs a) {
  Slot s;
  if (!slot_of(a, s)) return;
  const Packs P(a);
  const Planes E = planes_of(a);
  const double mk = P.X[s.k].w, dbk = P.DB[s.k];
  const uint32_t* __restrict__ my = a.nlist + list_base(s.k, a.cap);
  Sums sum = {{0, 0, 0}, {0, 0, 0}, 0, 0, 0};
  // all lanes at the same entry index, so the entry-plane loads coalesce (this pass waits on its
  // loads; starting each lane at its own first upper entry made it slower)
  for (uint32_t q = 0; q < s.L; ++q) {
    const uint32_t t = my[(size_t)q * kListTile];
    if (t < s.k) continue;
    const size_t e = entry(s.k, q, a.cap);
    const double D = dbk * E.at(kMt, e) + P.DB[t] * mk;
    double Vx[3] = {0, 0, 0}, Vv[3] = {0, 0, 0};
#pragma unroll
    for (int cc = 0; cc < DIM; ++cc) {
      Vx[cc] = D * E.at(kU1 + cc, e);
      Vv[cc] = D * E.at(kU2 + cc, e);
      sum.gx[cc] += Vx[cc];
      sum.gv[cc] += Vv[cc];
    }
    const uint32_t mt = E.mirror(e);
    if (mt != kNoMirror) {
      const size_t f = entry(t, mt, a.cap);
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) {
        E.at(kMx + cc, f) = Vx[cc];
        E.at(kMv + cc, f) = Vv[cc];
      }
    }
  }
  store_sums(a, P, s.k, sum, 6);
}

template <int DIM>
__global__ void __launch_bounds__(kSphMaxThreads) adj_c2_kernel(SphArgs a) {
  Slot s;
  if (!slot_of(a, s)) return;
  const SphK& K = a.sys[0];
  const Packs P(a);
  const Planes E = planes_of(a);
  const double4_32a xk = P.X[s.k], vk = P.V[s.k];
  const uint32_t* __restrict__ my = a.nlist + list_base(s.k, a.cap);
  Sums sum = load_sums(a, P, s.k, 6);
  const uint32_t below = first_above(my, s.L, s.k);
  for (uint32_t q = 0; q < below; ++q) {
    const uint32_t t = my[(size_t)q * kListTile];
    if (holds(a, t, s.k)) {
      const size_t e = entry(s.k, q, a.cap);
#pragma unroll
      for (int cc = 0; cc < DIM; ++cc) {
        sum.gx[cc] -= E.at(kMx + cc, e);
        sum.gv[cc] -= E.at(kMv + cc, e);
      }
    } else {
      cont_full<DIM>(K, P, s.k, t, xk, vk, sum);
    }
  }
  if (s.overflow) resume_walk<DIM>(a, K, P, s.k, xk, [&](uint32_t t) { cont_full<DIM>(K, P, s.k, t, xk, vk, sum); });
  double* lx = (double*)a.lam[0];
  double* lv = (double*)a.lam[1];
#pragma unroll
  for (int cc = 0; cc < DIM; ++cc) {
    const size_t o = (size_t)s.id * DIM + cc;
    lx[o] += sum.gx[cc];
    lv[o] += sum.gv[cc];
  }
}

typedef void (*AdjSymKernel)(SphArgs);

template <int DIM>
AdjSymKernel adj_sym_kernel(int part) {
  switch (part) {
    case 0: return adj_mirror_kernel;
    case 1: return adj_a1_kernel<DIM>;
    case 2: return adj_a2_kernel<DIM>;
    case 3: return adj_c1_kernel<DIM>;
    case 4: return adj_c2_kernel<DIM>;
    default: return nullptr;
  }
}

}  // namespace

size_t adjoint_sym_entry_bytes() { return kPlanes * sizeof(double) + sizeof(uint32_t); }
size_t adjoint_sym_slot_bytes() { return kSlotSums * sizeof(double); }

int launch_adjoint_sym(cudaStream_t st, const SphArgs& a, int part) {
  AdjSymKernel kern = a.dim == 2 ? adj_sym_kernel<2>(part) : adj_sym_kernel<3>(part);
  if (!kern) {
    set_error("unknown part %d of the pair-once adjoint", part);
    return PG_EINVAL;
  }
  if (a.n == 0) return PG_OK;
  kern<<<(a.n + kSphThreads - 1) / kSphThreads, kSphThreads, 0, st>>>(a);
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

}  // namespace pg
