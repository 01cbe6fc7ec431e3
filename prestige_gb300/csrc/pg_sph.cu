// Weakly-compressible SPH on the cell list: continuity, Tait pressure, Monaghan artificial
// viscosity and the symplectic Euler integrator.
//
// The reference states a pairwise equation as a gather into particle i over partners j
// (prestige/src/lib.rs:7-12 `force[i] += mass[j]`, executed by the loop of
// prestige/src/codegen/simple_cpu.rs:7-19).  These passes are that gather for the SPH rates,
// with j restricted to the particles of the neighbour cells and r_ij < 2h:
//   C_i = drho_i = sum_j m_j (v_ij . x_ij) F_ij
//   M_i = a_i    = -sum_j m_j (P_i + P_j + Pi_ij) F_ij x_ij           (+ g in the integrator)
//   F = (dW/dr)/r of the cubic spline (support 2h), P = p/rho^2, p = B((rho/rho0)^gamma - 1)
//   Pi_ij  = -2 alpha c0 h (v_ij.x_ij) / ((r^2 + eps h^2)(rho_i + rho_j))  if v_ij.x_ij < 0
//
// One time step is two passes over the same neighbour structure:
//   continuity pass  rho' = rho + dt C(x, v)   (writes rho' and P(rho') into the sorted pack)
//   momentum pass    v' = v + dt (M(x, v, rho') + g),  x' = x + dt v'   (fluid particles)
// Advancing the density first makes the acoustic pair (rho, v) symplectic; evaluating both
// rates from one snapshot would advance it by forward Euler, which amplifies every acoustic
// mode.  A third variant (pg_compute_rates) evaluates C and M of one state in one pass.
//
// Kernel structure (one thread per target particle i, slot order; pg_sph_pass.cuh):
//   phase 1  every candidate of the 9 (2D: 3) neighbour rows is tested in FP32 against a
//            conservative bound on r^2; passing slots are appended to a per-thread list in
//            shared memory.
//   phase 2  when any lane's list is full (or all lanes are done) the warp evaluates the
//            listed pairs: the exact neighbour test, then the pair terms.
// Pairs are evaluated in the oracle's order (rows z, y ascending; slots ascending), so the
// IEEE modes reproduce the oracle bit for bit.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pg_arith.cuh"
#include "pg_internal.cuh"
#include "pg_kernels.cuh"
#include "pg_sph_pass.cuh"

namespace pg {

namespace {

using namespace sphpass;

template <class R> struct V2;
template <> struct V2<double> { typedef double2 T; };
template <> struct V2<float> { typedef float2 T; };

template <class R> __device__ __forceinline__ typename V2<R>::T make2(R a, R b);
template <> __device__ __forceinline__ double2 make2<double>(double a, double b) { return make_double2(a, b); }
template <> __device__ __forceinline__ float2 make2<float>(float a, float b) { return make_float2(a, b); }

// ---------------------------------------------------------------------------------------
// Sorted gather: slot k <- particle sorted_id[k]; precomputes P = p / rho^2.
//   IEEE modes:   s0 {x, y, z, m}   s1 {vx, vy, vz, 0}   s2 {rho, P}   (f64: s3 float4 x)
// ---------------------------------------------------------------------------------------
template <class Ops, int DIM>
__global__ void sph_gather_real(SphArgs a) {
  typedef typename Ops::R R;
  typedef typename V4<R>::T R4;
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const uint32_t id = a.sorted_id[k];
  const SphK& K = a.sys[sys_of_slot(a, id)];
  const R* pos = (const R*)a.pos;
  const R* vel = (const R*)a.vel;
  const R rho = ((const R*)a.rho)[id];
  const R m = ((const R*)a.mass)[id];
  R x[3] = {0, 0, 0}, v[3] = {0, 0, 0};
#pragma unroll
  for (int c = 0; c < DIM; ++c) {
    x[c] = pos[(size_t)id * DIM + c];
    v[c] = vel[(size_t)id * DIM + c];
  }
  R4 A, B;
  A.x = x[0]; A.y = x[1]; A.z = x[2]; A.w = m;
  B.x = v[0]; B.y = v[1]; B.z = v[2]; B.w = R(0);
  ((R4*)a.s[0])[k] = A;
  ((R4*)a.s[1])[k] = B;
  ((typename V2<R>::T*)a.s[2])[k] = make2<R>(rho, tait_pterm<Ops>(consts<R>(K), K.gamma, rho));
  if (sizeof(R) == 8) ((float4*)a.s[3])[k] = make_float4((float)x[0], (float)x[1], (float)x[2], 0.f);
}

// Packs of the f64 fast (double-word) mode:
//   s0 {x,y,z,m}.hi (the list kernel's FP32 positions)
//   s1 DfRecord {x,y,z,m}.hi, {x,y,z,m}.lo, {vx,vy,vz,0}.hi, {vx,vy,vz,0}.lo (the pair passes)
//   s4 {rho.hi, rho.lo, P.hi, P.lo}   s5 double {x,y,z} for the exact neighbour test near 2h.
// Positions in s0 and s1 are shifted (see sph_gather_df).

// p / rho^2 of the Tait law in double-word arithmetic on the FP32 pipe (relative error about
// 1e-12: (rho/rho0)^gamma - 1 loses the digits its cancellation takes).
__device__ __forceinline__ df tait_pterm_df(const SphDF& w, int gamma, df rho) {
  const df rr = df_mul(rho, df_make(w.inv_rho0[0], w.inv_rho0[1]));
  df pw = rr;
  for (int e = 1; e < gamma; ++e) pw = df_mul(pw, rr);
  const df p = df_mul(df_make(w.B[0], w.B[1]), df_add_f(pw, -1.0f));
  return df_div(p, df_mul(rho, rho));
}

// The {rho, P/rho^2} pack of the double-word mode, from the f64 density, without FP64 work
// beyond the density itself.
__device__ __forceinline__ float4 df_pack_rho(const SphDF& w, int gamma, double rho) {
  float4 r;
  df_split_fast(rho, &r.x, &r.y);
  const df pt = tait_pterm_df(w, gamma, df_make(r.x, r.y));
  r.z = pt.hi;
  r.w = pt.lo;
  return r;
}

// The packed {rho', P'} of every slot from the canonical density, exactly as the continuity pass
// packs them (pg_step_stage: the caller may replace densities between the two passes).
template <class Ops>
__global__ void sph_repack_rho_real(SphArgs a) {
  typedef typename Ops::R R;
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const uint32_t id = a.sorted_id[k];
  const SphK& K = a.sys[sys_of_slot(a, id)];
  const R rn = ((const R*)a.rho)[id];
  ((typename V2<R>::T*)a.s[2])[k] = make2<R>(rn, tait_pterm<Ops>(consts<R>(K), K.gamma, rn));
}

__global__ void sph_repack_rho_df(SphArgs a) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const uint32_t id = a.sorted_id[k];
  const SphK& K = a.sys[sys_of_slot(a, id)];
  ((float4*)a.s[4])[k] = df_pack_rho(K.w, K.gamma, ((const double*)a.rho)[id]);
}

// The pair passes' per-slot record in the double-word mode: positions and mass (hi, lo) and
// velocities (hi, lo), 64 bytes, so the four loads of a neighbour touch two sectors of one line.
struct __align__(64) DfRecord {
  float4 ah, al, bh, bl;
};

// Packs of the double-word mode.  Positions in the record and in the FP32 array are shifted by
// pos_pad - min (per system and dimension, pos_pad = 8h of the system), so every packed coordinate
// is at least 8h: the hi parts of two particles closer than 2h are then within a factor 2 of each
// other and the pair passes take differences with df_sub_close.  The shift is common to all
// particles of a system (pairs never cross systems), so differences are unchanged up to one f64
// rounding of each shifted coordinate, and a system's packs, hence its results, do not depend on
// the other systems of a batch; the f64 array for the exact test keeps the unshifted positions.
template <int DIM>
__global__ void sph_gather_df(SphArgs a) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const uint32_t id = a.sorted_id[k];
  const uint32_t sys = sys_of_slot(a, id);
  const SphK& K = a.sys[sys];
  const double* pos = (const double*)a.pos;
  const double* vel = (const double*)a.vel;
  const double rho = ((const double*)a.rho)[id];
  const double m = ((const double*)a.mass)[id];
  double x[3] = {0, 0, 0}, v[3] = {0, 0, 0};
#pragma unroll
  for (int c = 0; c < DIM; ++c) {
    x[c] = pos[(size_t)id * DIM + c];
    v[c] = vel[(size_t)id * DIM + c];
  }
  double xs[3] = {K.pos_pad, K.pos_pad, K.pos_pad};
#pragma unroll
  for (int c = 0; c < DIM; ++c) xs[c] = __dadd_rn(__dsub_rn(x[c], ordered_value(a.posmin[3 * sys + c])), K.pos_pad);
  float4 ah, al, bh, bl;
  df_split_fast(xs[0], &ah.x, &al.x);
  df_split_fast(xs[1], &ah.y, &al.y);
  df_split_fast(xs[2], &ah.z, &al.z);
  df_split_fast(m, &ah.w, &al.w);
  df_split_fast(v[0], &bh.x, &bl.x);
  df_split_fast(v[1], &bh.y, &bl.y);
  df_split_fast(v[2], &bh.z, &bl.z);
  bh.w = bl.w = 0.f;
  ((float4*)a.s[0])[k] = ah;
  DfRecord rec;
  rec.ah = ah;
  rec.al = al;
  rec.bh = bh;
  rec.bl = bl;
  ((DfRecord*)a.s[1])[k] = rec;
  ((float4*)a.s[4])[k] = df_pack_rho(K.w, K.gamma, rho);
  ((double4_32a*)a.s[5])[k] = make_double4_32a(x[0], x[1], x[2], 0.0);
}

// ---------------------------------------------------------------------------------------
// Pair-term policies.  STAGE: SPH_RATES (C and M of one state, written to acc/drho),
// SPH_CONT (C, then rho' = rho + dt C into the canonical state and the sorted pack),
// SPH_MOM (M with the packed rho', then the velocity and position update).
// ---------------------------------------------------------------------------------------
template <class Ops, int DIM, bool EXACT_TEST, int STAGE>
struct RealPairs {
  typedef typename Ops::R R;
  typedef typename V4<R>::T R4;
  typedef typename V2<R>::T R2;
  static constexpr bool kCont = STAGE != SPH_MOM;
  static constexpr bool kMom = STAGE != SPH_CONT;
  const R4* A;
  const R4* B;
  const R2* Q;
  SphC<R> c;
  R xi[3], vi[3], rhoi, Pi;
  R acc[3], dr;

  __device__ __forceinline__ void begin(const SphArgs& a, const SphK& K, uint32_t k) {
    A = (const R4*)a.s[0];
    B = (const R4*)a.s[1];
    Q = (const R2*)a.s[2];
    c = consts<R>(K);
    const R4 Ai = A[k], Bi = B[k];
    xi[0] = Ai.x; xi[1] = Ai.y; xi[2] = Ai.z;
    vi[0] = Bi.x; vi[1] = Bi.y; vi[2] = Bi.z;
    rhoi = Pi = R(0);
    if (kMom) {
      const R2 q = Q[k];
      rhoi = q.x;
      Pi = q.y;
    }
    acc[0] = acc[1] = acc[2] = R(0);
    dr = R(0);
  }

  // The neighbour's pack records, loaded ahead of its pair terms.
  struct Pre {
    R4 a, b;
    R2 q;
  };
  static constexpr bool kPrefetch = true;

  __device__ __forceinline__ Pre fetch(uint32_t t, uint32_t) const {
    Pre p;
    p.a = A[t];
    p.b = B[t];
    if (kMom) p.q = Q[t];
    return p;
  }

  // A candidate of the continued walk of an overflowed list (a superset: EXACT_TEST repeats the
  // oracle's test).
  __device__ __forceinline__ void pair(uint32_t t) { terms<EXACT_TEST>(t, fetch(t, 0)); }

  // A list entry: the lists hold exactly the oracle's neighbours in every mode (f64 lists are
  // classified with the f64 test, f32 lists with the IEEE FP32 test), so no test is repeated.
  __device__ __forceinline__ void pair_with(uint32_t t, uint32_t, const Pre& p) { terms<false>(t, p); }

  template <bool TEST>
  __device__ __forceinline__ void terms(uint32_t t, const Pre& p) {
    const R4 Aj = p.a;
    const R d0 = Ops::sub(xi[0], Aj.x), d1 = Ops::sub(xi[1], Aj.y);
    const R d2 = DIM == 3 ? Ops::sub(xi[2], Aj.z) : R(0);
    R r2 = Ops::add(Ops::mul(d0, d0), Ops::mul(d1, d1));
    if (DIM == 3) r2 = Ops::add(r2, Ops::mul(d2, d2));
    if (TEST) {
      if (!(r2 < c.four_h2)) return;
      if (!(r2 > R(0))) return;
    }
    const R4 Bj = p.b;
    const R r = Ops::sqrt(r2);
    const R q = Ops::mul(r, c.inv_h);
    // both pieces of the spline in the oracle's operation order, then a select (no divergence;
    // the selected value is bit for bit the oracle's)
    const R tq = Ops::sub(R(2), q);
    const R Fnear = Ops::mul(c.fa, Ops::sub(Ops::mul(R(2.25), q), R(3)));
    const R Ffar = Ops::div(Ops::mul(c.fb, Ops::mul(tq, tq)), r);
    const R F = q < R(1) ? Fnear : Ffar;
    const R dv0 = Ops::sub(vi[0], Bj.x), dv1 = Ops::sub(vi[1], Bj.y);
    const R dv2 = DIM == 3 ? Ops::sub(vi[2], Bj.z) : R(0);
    R w = Ops::add(Ops::mul(dv0, d0), Ops::mul(dv1, d1));
    if (DIM == 3) w = Ops::add(w, Ops::mul(dv2, d2));
    const R mj = Aj.w;
    if (kCont) dr = Ops::add(dr, Ops::mul(mj, Ops::mul(w, F)));
    if (kMom) {
      const R2 qj = p.q;
      const R av = Ops::div(Ops::mul(c.avk, w), Ops::mul(Ops::add(r2, c.eps_h2), Ops::add(rhoi, qj.x)));
      const R pij = w < R(0) ? av : R(0);
      const R coef = Ops::mul(mj, Ops::mul(Ops::add(Ops::add(Pi, qj.y), pij), F));
      acc[0] = Ops::sub(acc[0], Ops::mul(coef, d0));
      acc[1] = Ops::sub(acc[1], Ops::mul(coef, d1));
      if (DIM == 3) acc[2] = Ops::sub(acc[2], Ops::mul(coef, d2));
    }
  }

  // Sum the partial sums of the LANES lanes of a slot (butterfly; every lane ends with the sum).
  template <int LANES>
  __device__ __forceinline__ void reduce_lanes() {
#pragma unroll
    for (int off = 1; off < LANES; off <<= 1) {
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) acc[cc] = Ops::add(acc[cc], __shfl_xor_sync(0xffffffffu, acc[cc], off));
      dr = Ops::add(dr, __shfl_xor_sync(0xffffffffu, dr, off));
    }
  }

  __device__ __forceinline__ void finish(const SphArgs& a, const SphK& K, uint32_t id, uint32_t k) {
    if (STAGE == SPH_RATES) {
#pragma unroll
      for (int cc = 0; cc < DIM; ++cc) ((R*)a.acc)[(size_t)id * DIM + cc] = acc[cc];
      ((R*)a.drho)[id] = dr;
    } else if (STAGE == SPH_CONT) {
      R* rho = (R*)a.rho;
      const R rn = Ops::add(rho[id], Ops::mul(c.dt, dr));
      rho[id] = rn;
      ((R2*)a.s[2])[k] = make2<R>(rn, tait_pterm<Ops>(c, K.gamma, rn));
    } else if (id < K.fluid_end) {
      R* pos = (R*)a.pos;
      R* vel = (R*)a.vel;
#pragma unroll
      for (int cc = 0; cc < DIM; ++cc) {
        const size_t o = (size_t)id * DIM + cc;
        const R v = Ops::add(vel[o], Ops::mul(c.dt, Ops::add(acc[cc], c.g[cc])));
        vel[o] = v;
        pos[o] = Ops::add(pos[o], Ops::mul(c.dt, v));
      }
    }
  }
};

template <int DIM, int STAGE>
struct DfPairs {
  static constexpr bool kCont = STAGE != SPH_MOM;
  static constexpr bool kMom = STAGE != SPH_CONT;
  const DfRecord* Rec;
  const float4* RP;
  const double4_32a* Xd;
  SphDF w;
  double four_h2;
  uint32_t kself;
  float4* fc;  // per list entry {G.hi, G.lo, u.hi, u.lo} with G = m_j F and u = w / (r^2 + eps h^2):
               // written by the continuity pass, read by the momentum pass
  df xi[3], vi[3], rhoi, Pi;
  dfacc acc[3], dr;
  static constexpr bool kCacheF = STAGE == SPH_CONT || STAGE == SPH_MOM;

  __device__ __forceinline__ void begin(const SphArgs& a, const SphK& K, uint32_t k) {
    Rec = (const DfRecord*)a.s[1];
    RP = (const float4*)a.s[4];
    Xd = (const double4_32a*)a.s[5];
    w = K.w;
    four_h2 = K.d.four_h2;
    const float4 ah = Rec[k].ah, al = Rec[k].al, bh = Rec[k].bh, bl = Rec[k].bl;
    xi[0] = df_make(ah.x, al.x); xi[1] = df_make(ah.y, al.y); xi[2] = df_make(ah.z, al.z);
    vi[0] = df_make(bh.x, bl.x); vi[1] = df_make(bh.y, bl.y); vi[2] = df_make(bh.z, bl.z);
    rhoi = Pi = df_make(0.f, 0.f);
    if (kMom) {
      const float4 rp = RP[k];
      rhoi = df_make(rp.x, rp.y);
      Pi = df_make(rp.z, rp.w);
    }
    kself = k;
    fc = kCacheF && a.fcache ? (float4*)a.fcache + list_base(k, a.cap) : nullptr;
    acc[0] = acc[1] = acc[2] = dfacc_zero();
    dr = dfacc_zero();
  }

  // Geometry of pair (k, t): x_ij, r^2, F = (dW/dr)/r and w = v_ij . x_ij.  CHECK: false when t is
  // not a neighbour (outside the support, or t == k), the oracle's f64 test deciding when the
  // double-word r^2 is within a relative band of 1e-9 of (2h)^2.  Without CHECK, t comes from an
  // exact neighbour list (sph_list_kernel with f64 classification).
  // The sorted-pack records of one neighbour, loaded ahead of its pair terms.
  struct Pre {
    float4 ah, al, bh, bl, rp, fw;
  };
  static constexpr bool kPrefetch = true;

  __device__ __forceinline__ Pre fetch(uint32_t t, uint32_t q) const { return fetch_entry(t, q, STAGE == SPH_MOM && fc); }

  // the momentum pass's cache entries are a DRAM stream like the lists (sph_list_pass_kernel)
  static constexpr bool kL2Entry = STAGE == SPH_MOM;
  __device__ __forceinline__ void prefetch_entry(uint32_t q) const {
    if (fc) prefetch_l2(fc + (size_t)q * kListTile);
  }

  // cached: list entry q of a momentum pass that reads G = m_j F and u from the continuity pass
  __device__ __forceinline__ Pre fetch_entry(uint32_t t, uint32_t q, bool cached) const {
    Pre p;
    p.ah = Rec[t].ah;
    p.al = Rec[t].al;
    // the momentum pass takes w from the cache and needs no velocities of the neighbour
    p.bh = cached ? make_float4(0.f, 0.f, 0.f, 0.f) : Rec[t].bh;
    p.bl = cached ? make_float4(0.f, 0.f, 0.f, 0.f) : Rec[t].bl;
    p.rp = kMom ? RP[t] : make_float4(0.f, 0.f, 0.f, 0.f);
    p.fw = cached ? fc[q * kListTile] : make_float4(0.f, 0.f, 0.f, 0.f);
    return p;
  }

  // CACHED: F holds G = m_j F and wv holds u = w / (r^2 + eps h^2), both from the continuity pass
  // (list entries of a step's momentum pass); r2 is then not computed: the continuity pass wrote
  // a zero entry for a listed pair it skipped (coincident double-word positions).
  template <bool CHECK, bool CACHED = false>
  __device__ __forceinline__ bool geometry(uint32_t t, const Pre& p, df* d, df& r2, df& F, df& wv, df& mj) const {
    const float4 ah = p.ah, al = p.al;
    d[0] = df_sub_close(xi[0], df_make(ah.x, al.x));
    d[1] = df_sub_close(xi[1], df_make(ah.y, al.y));
    d[2] = DIM == 3 ? df_sub_close(xi[2], df_make(ah.z, al.z)) : df_make(0.f, 0.f);
    r2 = df_make(0.f, 0.f);
    if (!CACHED) {
      r2 = df_sumsq3(d[0], d[1], d[2]);
      if (CHECK) {
        const df gap = df_sub(r2, df_make(w.four_h2[0], w.four_h2[1]));
        if (fabsf(gap.hi) <= w.band) {
          if (!exact_neighbor_call<DIM>(Xd, kself, t, four_h2)) return false;
        } else if (!(gap.hi < 0.f)) {
          return false;
        }
      }
      if (!(r2.hi > 0.f)) return false;
    }
    if (CACHED) {
      F = df_make(p.fw.x, p.fw.y);
    } else {
      const df inv_r = df_rsqrt(r2);
      // F = c0 + c1 r + c2 / r = c0 + (c1 r^2 + c2) / r on either piece of the spline, without a
      // branch and without forming r (F is continuous at r = h, so the piece chosen by the FP32
      // r^2 there does not matter beyond rounding)
      const bool near = r2.hi < w.h2;
      const df c0 = near ? df_make(w.near0[0], w.near0[1]) : df_make(w.far0[0], w.far0[1]);
      const df c1 = near ? df_make(w.near1[0], w.near1[1]) : df_make(w.far1[0], w.far1[1]);
      const df c2 = near ? df_make(0.f, 0.f) : df_make(w.far2[0], w.far2[1]);
      F = df_add_raw(c0, df_mul(df_add_raw(df_mul(c1, r2), c2), inv_r));  // consumed by products
    }
    if (CACHED) {
      wv = df_make(p.fw.z, p.fw.w);
    } else {
      const float4 bh = p.bh, bl = p.bl;
      // velocity differences, consumed by the dot product only
      const df dv0 = df_sub_raw(vi[0], df_make(bh.x, bl.x));
      const df dv1 = df_sub_raw(vi[1], df_make(bh.y, bl.y));
      const df dv2 = DIM == 3 ? df_sub_raw(vi[2], df_make(bh.z, bl.z)) : df_make(0.f, 0.f);
      wv = df_dot3(dv0, dv1, dv2, d[0], d[1], d[2]);
    }
    mj = df_make(ah.w, al.w);
    return true;
  }

  // u = w / (r^2 + eps h^2), the velocity factor of the artificial viscosity, with the sign of w
  __device__ __forceinline__ df visc_u(df r2, df wv) const {
    return df_div(wv, df_add_raw(r2, df_make(w.eps_h2[0], w.eps_h2[1])));  // a sum of positive terms
  }

  // G = m_j F and u (computed here, or from the cache)
  __device__ __forceinline__ void momentum(const float4& rpj, const df* d, df G, df u) {
    // artificial viscosity where the pair approaches (w < 0, so u < 0), computed for every pair
    // and then selected: nearly every warp has lanes on both sides
    const df den = df_add_raw(rhoi, df_make(rpj.x, rpj.y));  // a sum of positive terms
    const df av = df_div(df_mul(df_make(w.avk[0], w.avk[1]), u), den);
    const df pij = u.hi < 0.f ? av : df_make(0.f, 0.f);
    const df ncoef = df_neg(df_mul(df_add_raw(df_add_raw(Pi, df_make(rpj.z, rpj.w)), pij), G));
    dfacc_add_prod(acc[0], ncoef, d[0]);
    dfacc_add_prod(acc[1], ncoef, d[1]);
    if (DIM == 3) dfacc_add_prod(acc[2], ncoef, d[2]);
  }

  template <bool CHECK, bool CACHED>
  __device__ __forceinline__ void terms(uint32_t t, uint32_t q, const Pre& p) {
    constexpr bool kStore = STAGE == SPH_CONT && !CHECK;  // list entries of the continuity pass
    df d[3], r2, F, wv, mj;
    if (!geometry<CHECK, CACHED>(t, p, d, r2, F, wv, mj)) {
      if (kStore && fc) fc[q * kListTile] = make_float4(0.f, 0.f, 0.f, 0.f);  // contributes nothing
      return;
    }
    const df G = CACHED ? F : df_mul(mj, F);
    if (kStore && fc) {
      const df u = visc_u(r2, wv);
      fc[q * kListTile] = make_float4(G.hi, G.lo, u.hi, u.lo);
    }
    if (kCont) dfacc_add_prod(dr, G, wv);
    if (kMom) momentum(p.rp, d, G, CACHED ? wv : visc_u(r2, wv));
  }

  // entry q of an exact neighbour list
  __device__ __forceinline__ void pair_with(uint32_t t, uint32_t q, const Pre& p) {
    if (STAGE == SPH_MOM && fc) terms<false, true>(t, q, p);
    else terms<false, false>(t, q, p);
  }
  // any candidate (the walk that continues an overflowed list): everything computed here
  __device__ __forceinline__ void pair(uint32_t t) { terms<true, false>(t, 0, fetch_entry(t, 0, false)); }

  // Combine the partial sums of the LANES lanes of a slot (butterfly; every lane ends with the sum).
  template <int LANES>
  __device__ __forceinline__ void reduce_lanes() {
#pragma unroll
    for (int off = 1; off < LANES; off <<= 1) {
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) {
        dfacc o;
        o.hi = __shfl_xor_sync(0xffffffffu, acc[cc].hi, off);
        o.lo = __shfl_xor_sync(0xffffffffu, acc[cc].lo, off);
        acc[cc] = dfacc_add(acc[cc], o);
      }
      dfacc o;
      o.hi = __shfl_xor_sync(0xffffffffu, dr.hi, off);
      o.lo = __shfl_xor_sync(0xffffffffu, dr.lo, off);
      dr = dfacc_add(dr, o);
    }
  }

  __device__ __forceinline__ void finish(const SphArgs& a, const SphK& K, uint32_t id, uint32_t k) {
    const SphC<double>& c = K.d;
    if (STAGE == SPH_RATES) {
#pragma unroll
      for (int cc = 0; cc < DIM; ++cc) ((double*)a.acc)[(size_t)id * DIM + cc] = dfacc_to_double(acc[cc]);
      ((double*)a.drho)[id] = dfacc_to_double(dr);
    } else if (STAGE == SPH_CONT) {
      double* rho = (double*)a.rho;
      const double rn = __dadd_rn(rho[id], __dmul_rn(c.dt, dfacc_to_double(dr)));
      rho[id] = rn;
      ((float4*)a.s[4])[k] = df_pack_rho(K.w, K.gamma, rn);
    } else if (id < K.fluid_end) {
      double* pos = (double*)a.pos;
      double* vel = (double*)a.vel;
#pragma unroll
      for (int cc = 0; cc < DIM; ++cc) {
        const size_t o = (size_t)id * DIM + cc;
        const double v = __dadd_rn(vel[o], __dmul_rn(c.dt, __dadd_rn(dfacc_to_double(acc[cc]), c.g[cc])));
        vel[o] = v;
        pos[o] = __dadd_rn(pos[o], __dmul_rn(c.dt, v));
      }
    }
  }
};

// ---------------------------------------------------------------------------------------
// Launch plumbing: one table of kernel instantiations per (arith, dim, stage).
// ---------------------------------------------------------------------------------------
typedef void (*PassKernel)(SphArgs, int);

// Kernel table for the list-based passes and the list kernel (stage < 0).
template <int DIM, int STAGE, int LANES>
PassKernel list_pass_lanes(int arith, int* pf_index) {
  *pf_index = 0;
  switch (arith) {
    case ARITH_F64_DF: return sph_list_pass_kernel<DfPairs<DIM, STAGE>, DIM, false, LANES>;
    case ARITH_F32_FAST: return sph_list_pass_kernel<RealPairs<OpsFF, DIM, false, STAGE>, DIM, true, LANES>;
    default: return nullptr;
  }
}

template <int DIM, int STAGE>
PassKernel list_pass_for(int arith, int* pf_index, int lanes) {
  if (lanes == 2) return list_pass_lanes<DIM, STAGE, 2>(arith, pf_index);
  if (lanes == 4) return list_pass_lanes<DIM, STAGE, 4>(arith, pf_index);
  switch (arith) {
    case ARITH_F64_EXACT:
      *pf_index = 3;
      return sph_list_pass_kernel<RealPairs<OpsD, DIM, true, STAGE>, DIM, false>;
    case ARITH_F64_DF:
      *pf_index = 0;
      return sph_list_pass_kernel<DfPairs<DIM, STAGE>, DIM, false>;
    case ARITH_F32_EXACT:
      *pf_index = 0;
      return sph_list_pass_kernel<RealPairs<OpsF, DIM, false, STAGE>, DIM, true>;
    case ARITH_F32_FAST:
      *pf_index = 0;
      return sph_list_pass_kernel<RealPairs<OpsFF, DIM, false, STAGE>, DIM, true>;
    default:
      return nullptr;
  }
}

template <int DIM>
PassKernel list_kernel_dim(int arith, int stage, int lanes, int* pf_index) {
  switch (stage) {
    case SPH_RATES: return list_pass_for<DIM, SPH_RATES>(arith, pf_index, 1);
    case SPH_CONT: return list_pass_for<DIM, SPH_CONT>(arith, pf_index, lanes);
    case SPH_MOM: return list_pass_for<DIM, SPH_MOM>(arith, pf_index, lanes);
    default: break;
  }
  switch (arith) {  // the list kernel
    case ARITH_F64_EXACT:  // exact lists (FP32 prefilter, the f64 test in the band): the passes skip the test
      *pf_index = 3;
      return sph_list_kernel<DIM, false, 0>;
    case ARITH_F64_DF:  // exact lists: the double-word passes skip the neighbour test
      *pf_index = 0;
      return sph_list_kernel<DIM, false, 5>;
    case ARITH_F32_EXACT:
    case ARITH_F32_FAST:
      *pf_index = 0;
      return sph_list_kernel<DIM, true, -1>;
    default:
      return nullptr;
  }
}

PassKernel list_kernel(int arith, int dim, int stage, int lanes, int* pf_index) {
  lanes = sph_pass_lanes(arith, stage, lanes);
  return dim == 2 ? list_kernel_dim<2>(arith, stage, lanes, pf_index)
                  : list_kernel_dim<3>(arith, stage, lanes, pf_index);
}

// lanes: threads per slot of the kernel (1 for the list kernel); a block covers block / lanes slots.
int launch_table(cudaStream_t st, const SphArgs& a, PassKernel kern, int pf, int grid, int block, int lanes) {
  if (!kern) {
    set_error("unknown arithmetic mode or stage");
    return PG_EINVAL;
  }
  if (block < 32 || block > kSphMaxThreads || block % 32) {
    set_error("block size %d must be a multiple of 32 in 32..%d", block, kSphMaxThreads);
    return PG_EINVAL;
  }
  if (a.k_begin % (uint32_t)block || a.k_end > a.n || a.k_begin > a.k_end) {
    set_error("slot range [%u, %u) does not fit block size %d and n = %u", a.k_begin, a.k_end, block, a.n);
    return PG_EINVAL;
  }
  if (a.k_end == a.k_begin) return PG_OK;
  const uint32_t spb = (uint32_t)(block / lanes);
  const uint32_t ntiles = (a.k_end + spb - 1) / spb - a.k_begin / spb;
  if (grid <= 0 || (uint32_t)grid > ntiles) grid = (int)ntiles;
  kern<<<grid, block, 0, st>>>(a, pf);
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

}  // namespace

void sph_sorted_layout(int arith, size_t sz[6]) {
  for (int i = 0; i < 6; ++i) sz[i] = 0;
  switch (arith) {
    case ARITH_F64_EXACT:  // double4 {x,m}, double4 {v,0}, double2 {rho,P}, float4 prefilter positions
      sz[0] = 32; sz[1] = 32; sz[2] = 16; sz[3] = 16;
      break;
    case ARITH_F64_DF:  // float4 A.hi (list kernel), DfRecord {A.hi, A.lo, V.hi, V.lo} (pair passes),
                        // float4 {rho, P} (hi, lo), double4 exact positions
      sz[0] = 16; sz[1] = 64; sz[4] = 16; sz[5] = 32;
      break;
    default:  // float4 {x,m}, float4 {v,0}, float2 {rho,P}
      sz[0] = 16; sz[1] = 16; sz[2] = 8;
      break;
  }
}

int launch_sph_gather(cudaStream_t st, const SphArgs& a, int arith) {
  if (a.n == 0) return PG_OK;
  const unsigned blocks = (a.n + 255) / 256;
  const int dim = a.dim;
  switch (arith) {
    case ARITH_F64_EXACT:
      if (dim == 2) sph_gather_real<OpsD, 2><<<blocks, 256, 0, st>>>(a);
      else sph_gather_real<OpsD, 3><<<blocks, 256, 0, st>>>(a);
      break;
    case ARITH_F64_DF:  // a.posmin was filled by the step's hash kernel
      if (dim == 2) sph_gather_df<2><<<blocks, 256, 0, st>>>(a);
      else sph_gather_df<3><<<blocks, 256, 0, st>>>(a);
      break;
    case ARITH_F32_EXACT:
      if (dim == 2) sph_gather_real<OpsF, 2><<<blocks, 256, 0, st>>>(a);
      else sph_gather_real<OpsF, 3><<<blocks, 256, 0, st>>>(a);
      break;
    case ARITH_F32_FAST:
      if (dim == 2) sph_gather_real<OpsFF, 2><<<blocks, 256, 0, st>>>(a);
      else sph_gather_real<OpsFF, 3><<<blocks, 256, 0, st>>>(a);
      break;
    default:
      set_error("unknown arithmetic mode %d", arith);
      return PG_EINVAL;
  }
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

int sph_pass_lanes(int arith, int stage, int lanes) {
  const bool tolerant = arith == ARITH_F64_DF || arith == ARITH_F32_FAST;
  return tolerant && (stage == SPH_CONT || stage == SPH_MOM) && (lanes == 2 || lanes == 4) ? lanes : 1;
}

int launch_sph_repack_rho(cudaStream_t st, const SphArgs& a, int arith) {
  if (a.n == 0) return PG_OK;
  const unsigned blocks = (a.n + 255) / 256;
  switch (arith) {
    case ARITH_F64_EXACT: sph_repack_rho_real<OpsD><<<blocks, 256, 0, st>>>(a); break;
    case ARITH_F64_DF: sph_repack_rho_df<<<blocks, 256, 0, st>>>(a); break;
    case ARITH_F32_EXACT: sph_repack_rho_real<OpsF><<<blocks, 256, 0, st>>>(a); break;
    case ARITH_F32_FAST: sph_repack_rho_real<OpsFF><<<blocks, 256, 0, st>>>(a); break;
    default:
      set_error("unknown arithmetic mode %d", arith);
      return PG_EINVAL;
  }
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

int launch_sph_list(cudaStream_t st, const SphArgs& a, int arith, int grid, int block) {
  int pf = 0;
  PassKernel kern = list_kernel(arith, a.dim, -1, 1, &pf);
  return launch_table(st, a, kern, pf, grid, block, 1);
}

int launch_sph_list_pf(cudaStream_t st, const SphArgs& a, int pf_index, int grid, int block) {
  PassKernel kern = a.dim == 2 ? sph_list_kernel<2, false, -1> : sph_list_kernel<3, false, -1>;
  return launch_table(st, a, kern, pf_index, grid, block, 1);
}

int launch_sph_list_exact(cudaStream_t st, const SphArgs& a, int pf_index, int grid, int block) {
  PassKernel kern = a.dim == 2 ? sph_list_kernel<2, false, 0> : sph_list_kernel<3, false, 0>;
  return launch_table(st, a, kern, pf_index, grid, block, 1);
}

int launch_sph_list_pass(cudaStream_t st, const SphArgs& a, int arith, int stage, int grid, int block, int lanes) {
  int pf = 0;
  lanes = sph_pass_lanes(arith, stage, lanes);
  PassKernel kern = list_kernel(arith, a.dim, stage, lanes, &pf);
  return launch_table(st, a, kern, pf, grid, block, lanes);
}

int sph_list_regs(int arith, int dim, int stage, int lanes) {
  int pf = 0;
  PassKernel kern = list_kernel(arith, dim, stage, lanes, &pf);
  cudaFuncAttributes attr;
  if (!kern || cudaFuncGetAttributes(&attr, kern) != cudaSuccess) return 0;
  return attr.numRegs;
}

int sph_list_occupancy(int arith, int dim, int stage, int block, int lanes) {
  int pf = 0, blocks = 0;
  PassKernel kern = list_kernel(arith, dim, stage, lanes, &pf);
  if (!kern) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, block, 0) != cudaSuccess) return 0;
  return blocks;
}

}  // namespace pg
