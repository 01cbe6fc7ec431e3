// Reverse-mode differentiation of the SPH step (f64), with checkpointed recomputation.
//
// The reference has no differentiation; this is the adjoint of the forward step in pg_sph.cu
// (continuity, Tait pressure and Monaghan viscosity as gathers into i over neighbours j, the
// semantics of prestige/src/codegen/simple_cpu.rs:7-19, with the symplectic Euler update).
//
// Forward step t -> t+1 (fluid particles; wall particles keep x and v):
//   rho' = rho + dt C(x, v),   v' = v + dt (M(x, v, rho') + g),   x' = x + dt v'
// Given the adjoints (lx', lv', lr') of the state after the step:
//   momentum adjoint    abar = dt (lv' + dt lx')  (fluid; 0 for walls)
//                       Phi_M = sum_i abar_i . M_i,   lr'_tot = lr' + dPhi_M/drho'
//   continuity adjoint  dbar = dt lr'_tot,  Phi_C = sum_i dbar_i C_i
//   lx = lx' + dPhi_M/dx + dPhi_C/dx,   lv = (lv' + dt lx' | lv') + dPhi_M/dv + dPhi_C/dv,
//   lr = lr'_tot (C does not depend on rho)
// For one unordered pair (i, j) the two ordered terms of Phi combine, because x_ji = -x_ij,
// v_ji = -v_ij and w, F, Pi_ij, P_i + P_j are symmetric, into
//   Lam_M = -F S (x . E),  E = m_j abar_i - m_i abar_j,  S = P_i + P_j + Pi,  Pi = c1 w (w < 0)
//   Lam_C =  F w D,        D = dbar_i m_j + dbar_j m_i
//   x = x_i - x_j,  v = v_i - v_j,  w = v . x,  c1 = avk / ((r^2 + eps h^2)(rho_i + rho_j)),
//   F = (dW/dr)/r,  G = (dF/dr)/r
// whose derivatives give particle i's share without any scatter:
//   dLam_M/dx = [-G S xE + 2 F xE Pi / (r^2 + eps h^2)] x - F c1 xE v - F S E,
//   dLam_M/dv = -F c1 xE x,   dLam_M/drho_i = -F xE (P'(rho_i) - Pi / (rho_i + rho_j)),
//   dLam_C/dx = G w D x + F D v,   dLam_C/dv = F D x
// with xE = x . E and P'(rho) = B ((gamma - 2)(rho/rho0)^gamma + 2) / rho^3 (all densities
// are rho', the ones the momentum rate used).  The mixed-precision adjoint (below) evaluates Lam
// for all of a thread's neighbours, so the transpose of the pair Jacobian is a second gather
// over the same cell lists (no atomics, deterministic order); the FP64 adjoint
// (pg_adjoint_sym.cu) evaluates each pair once and writes the partner's share, the negated
// vectors, into the partner's list entry.  The parameter derivatives are the derivatives of
// Lam_M per unordered pair, each side taking half of every pair it evaluates:
//   dPhi/dalpha += -1/2 F xE (-2 c0 h) w / ((r^2 + eps h^2)(rho_i + rho_j))   (w < 0)
//   dPhi/dB     += -1/2 F xE (P_i + P_j) / B
// In this form the cancellation between the two ordered terms is done analytically inside E;
// summing m_j F (abar_i . x_ij)(P_i + P_j) over j instead cancels across neighbours and loses
// digits.  The per-particle sums are added in a fixed order at the end.
//
// Checkpointing: pg_forward_checkpointed keeps the state every `every` steps.  pg_backward
// walks the segments last to first; for each it restores the checkpoint, re-runs the forward
// steps while keeping each step's state, its updated density and its neighbour structure
// (sorted cells, sorted ids, cell table: integer data, reused as is), then sweeps the adjoint
// back through the segment.  The recompute of the previous segment runs beside the sweep (the
// handle's stream and a second one), so two segments are held.  Memory: (nsteps / every)
// checkpoints plus two segments.  An IEEE handle recomputes in the double-word mode (see
// RecomputeMode below).
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "pg_arith.cuh"
#include "pg_internal.cuh"
#include "pg_kernels.cuh"
#include "pg_sph_pass.cuh"
#include "pg_system.cuh"

struct pg_adjoint {
  int nsteps = 0, every = 0, nseg = 0;
  bool have_forward = false;
  size_t state_doubles = 0;  // n * (2 dim + 1): pos, vel, rho
  pg::DevBuf ckpt;           // nseg states
  pg::DevBuf final_state;
  // two segments' recomputed steps: one is swept (on `sweep`) while the previous segment is
  // recomputed into the other (on the handle's stream)
  pg::DevBuf seg_state[2];   // `every` states of a segment
  pg::DevBuf seg_rnext[2];   // rho' of each step of the segment
  pg::DevBuf seg_cell[2], seg_id[2], seg_start[2];
  pg::DevBuf nlist, nlen, nresume;  // the sweep's neighbour lists (the recompute uses the handle's)
  cudaStream_t sweep = nullptr;
  cudaEvent_t ev_rec[2] = {nullptr, nullptr}, ev_sweep[2] = {nullptr, nullptr};
  ~pg_adjoint() {
    if (sweep) {
      cudaStreamSynchronize(sweep);
      cudaStreamDestroy(sweep);
    }
    for (int b = 0; b < 2; ++b) {
      if (ev_rec[b]) cudaEventDestroy(ev_rec[b]);
      if (ev_sweep[b]) cudaEventDestroy(ev_sweep[b]);
    }
  }
  pg::DevBuf lx, lv, lr, ga, gb;
  pg::DevBuf X4, V4, Q4, A4, PF, DB;  // slot-ordered packs of one adjoint step
  pg::DevBuf EP, PS;                  // FP64 adjoint: per-entry pair values, per-slot partial sums
  int pass_grid[3] = {0, 0, 0};
  int pass_grid_fp32 = -1;
  size_t bytes() const {
    const pg::DevBuf* b[] = {&ckpt,         &final_state,  &seg_state[0], &seg_rnext[0], &seg_cell[0],
                             &seg_id[0],    &seg_start[0], &seg_state[1], &seg_rnext[1], &seg_cell[1],
                             &seg_id[1],    &seg_start[1], &nlist,        &nlen,         &nresume,
                             &lx,           &lv,           &lr,           &ga,           &gb,
                             &X4,           &V4,           &Q4,           &A4,           &PF,
                             &DB,           &EP,           &PS};
    size_t t = 0;
    for (const pg::DevBuf* d : b) t += d->bytes;
    return t;
  }
};

size_t pg_system::adjoint_bytes() const { return adj ? adj->bytes() : 0; }

namespace pg {

void destroy_adjoint(pg_system* s) {
  delete s->adj;
  s->adj = nullptr;
}

namespace {

using namespace sphpass;

// Slot-ordered packs for one adjoint step (a.rho points at rho' of the step):
//   X4 {x, y, z, m}   V4 {vx, vy, vz, rho'}   Q4 {P, P'(rho'), P/B, 0}   A4 {abar, 0}   PF float4 x
template <int DIM>
__global__ void adjoint_prep_kernel(SphArgs a) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const uint32_t id = a.sorted_id[k];
  const SphK& K = a.sys[0];
  const double* pos = (const double*)a.pos;
  const double* vel = (const double*)a.vel;
  const double* lx = (const double*)a.lam[0];
  const double* lv = (const double*)a.lam[1];
  const double rho = ((const double*)a.rho)[id];
  const double m = ((const double*)a.mass)[id];
  const double dt = K.d.dt;
  const bool fluid = id < K.fluid_end;
  double x[3] = {0, 0, 0}, v[3] = {0, 0, 0}, ab[3] = {0, 0, 0};
#pragma unroll
  for (int c = 0; c < DIM; ++c) {
    const size_t o = (size_t)id * DIM + c;
    x[c] = pos[o];
    v[c] = vel[o];
    ab[c] = fluid ? dt * (lv[o] + dt * lx[o]) : 0.0;
  }
  const double rr = rho * K.d.inv_rho0;
  double pw = rr;
  for (int e = 1; e < K.gamma; ++e) pw *= rr;
  const double inv_r2 = 1.0 / (rho * rho);
  const double P = tait_pterm<OpsD>(K.d, K.gamma, rho);
  const double Pd = K.d.B * ((double)(K.gamma - 2) * pw + 2.0) * inv_r2 / rho;
  const double PB = (pw - 1.0) * inv_r2;
  ((double4_32a*)a.s[0])[k] = make_double4_32a(x[0], x[1], x[2], m);
  ((double4_32a*)a.s[1])[k] = make_double4_32a(v[0], v[1], v[2], rho);
  ((double4_32a*)a.s[2])[k] = make_double4_32a(P, Pd, PB, 0.0);
  ((double4_32a*)a.s[3])[k] = make_double4_32a(ab[0], ab[1], ab[2], 0.0);
  ((float4*)a.s[4])[k] = make_float4((float)x[0], (float)x[1], (float)x[2], 0.f);
}

// ---------------------------------------------------------------------------------------
// Mixed-precision adjoint (handles in the fast f64 mode).  Positions and velocities are packed
// as FP32 (hi, lo) pairs, so the differences x_i - x_j and v_i - v_j keep FP32 relative
// accuracy despite the cancellation; every other factor and the pair derivatives are FP32; the
// adjoint state and the parameter sums stay double.
//   s0 {x.hi, y.hi, z.hi, m} (also the prefilter positions)   s1 {x.lo, y.lo, z.lo, 0}
//   s2 {vx.hi, vy.hi, vz.hi, rho'}   s3 {vx.lo, vy.lo, vz.lo, 0}   s4 {P, P', P/B, 0}
//   s5 {abar, 0}   s6 float dbar
// Per-particle sums (adjoint increments and parameter terms) use Kahan compensation.
// ---------------------------------------------------------------------------------------
// Sign of w = v_ij . x_ij from the double-word (hi, lo) records, evaluated in double: true if
// the pair approaches.  Out of line: only pairs whose FP32 w is within rounding of zero call it.
// (The records are loaded again here, one component at a time, rather than passed, which keeps
// the caller's registers.)
template <int DIM>
__device__ __noinline__ bool approaches_f64(const float4* XH, const float4* XL, const float4* VH, const float4* VL,
                                            uint32_t k, uint32_t t) {
  const float *xh = (const float*)XH, *xl = (const float*)XL, *vh = (const float*)VH, *vl = (const float*)VL;
  double w = 0.0;
#pragma unroll 1
  for (int c = 0; c < DIM; ++c) {
    const size_t i = 4 * (size_t)k + c, j = 4 * (size_t)t + c;
    const double d = ((double)xh[i] - (double)xh[j]) + ((double)xl[i] - (double)xl[j]);
    const double dv = ((double)vh[i] - (double)vh[j]) + ((double)vl[i] - (double)vl[j]);
    w = fma(dv, d, w);
  }
  return w < 0.0;
}

template <int DIM>
__global__ void adjoint_prep_f_kernel(SphArgs a) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const uint32_t id = a.sorted_id[k];
  const SphK& K = a.sys[0];
  const double* pos = (const double*)a.pos;
  const double* vel = (const double*)a.vel;
  const double* lx = (const double*)a.lam[0];
  const double* lv = (const double*)a.lam[1];
  const double rho = ((const double*)a.rho)[id];
  const double m = ((const double*)a.mass)[id];
  const double dt = K.d.dt;
  const bool fluid = id < K.fluid_end;
  float hx[3] = {0.f, 0.f, 0.f}, lxs[3] = {0.f, 0.f, 0.f}, hv[3] = {0.f, 0.f, 0.f}, lvs[3] = {0.f, 0.f, 0.f};
  float ab[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int c = 0; c < DIM; ++c) {
    const size_t o = (size_t)id * DIM + c;
    df_split(pos[o], &hx[c], &lxs[c]);
    df_split(vel[o], &hv[c], &lvs[c]);
    ab[c] = fluid ? (float)(dt * (lv[o] + dt * lx[o])) : 0.f;
  }
  const double rr = rho * K.d.inv_rho0;
  double pw = rr;
  for (int e = 1; e < K.gamma; ++e) pw *= rr;
  const double inv_r2 = 1.0 / (rho * rho);
  const double P = tait_pterm<OpsD>(K.d, K.gamma, rho);
  const double Pd = K.d.B * ((double)(K.gamma - 2) * pw + 2.0) * inv_r2 / rho;
  const double PB = (pw - 1.0) * inv_r2;
  ((float4*)a.s[0])[k] = make_float4(hx[0], hx[1], hx[2], (float)m);
  ((float4*)a.s[1])[k] = make_float4(lxs[0], lxs[1], lxs[2], 0.f);
  ((float4*)a.s[2])[k] = make_float4(hv[0], hv[1], hv[2], (float)rho);
  ((float4*)a.s[3])[k] = make_float4(lvs[0], lvs[1], lvs[2], 0.f);
  ((float4*)a.s[4])[k] = make_float4((float)P, (float)Pd, (float)PB, 0.f);
  ((float4*)a.s[5])[k] = make_float4(ab[0], ab[1], ab[2], 0.f);
}

template <int DIM, int STAGE>
struct AdjPairsF {
  static constexpr bool kMom = STAGE == SPH_MOM;
  const float4 *XH, *XL, *VH, *VL, *Q, *A;
  const float* DBp;
  float fa, fb, inv_h, four_h2, eps_h2, avk, avk_alpha;
  float xh[3], xl[3], vh[3], vl[3], ai[3], rhoi, mi, Pi, Pdi, PBi, dbi;
  float gx[3], gv[3], gr, gal, gB;
  float cx[3], cv[3], cr, ca, cb;  // compensation terms (Kahan summation)
  uint32_t kself;

  __device__ __forceinline__ void begin(const SphArgs& a, const SphK& K, uint32_t k) {
    kself = k;
    XH = (const float4*)a.s[0];
    XL = (const float4*)a.s[1];
    VH = (const float4*)a.s[2];
    VL = (const float4*)a.s[3];
    Q = (const float4*)a.s[4];
    A = (const float4*)a.s[5];
    DBp = (const float*)a.s[6];
    fa = (float)K.d.fa;
    fb = (float)K.d.fb;
    inv_h = (float)K.d.inv_h;
    four_h2 = (float)K.d.four_h2;
    eps_h2 = (float)K.d.eps_h2;
    avk = (float)K.d.avk;
    avk_alpha = (float)K.avk_alpha;
    const float4 x = XH[k], x2 = XL[k], v = VH[k], v2 = VL[k];
    xh[0] = x.x; xh[1] = x.y; xh[2] = x.z; mi = x.w;
    xl[0] = x2.x; xl[1] = x2.y; xl[2] = x2.z;
    vh[0] = v.x; vh[1] = v.y; vh[2] = v.z; rhoi = v.w;
    vl[0] = v2.x; vl[1] = v2.y; vl[2] = v2.z;
    Pi = Pdi = PBi = dbi = 0.f;
    ai[0] = ai[1] = ai[2] = 0.f;
    if (kMom) {
      const float4 q = Q[k], ab = A[k];
      Pi = q.x; Pdi = q.y; PBi = q.z;
      ai[0] = ab.x; ai[1] = ab.y; ai[2] = ab.z;
    } else {
      dbi = DBp[k];
    }
    gx[0] = gx[1] = gx[2] = 0.f;
    gv[0] = gv[1] = gv[2] = 0.f;
    cx[0] = cx[1] = cx[2] = 0.f;
    cv[0] = cv[1] = cv[2] = 0.f;
    gr = gal = gB = cr = ca = cb = 0.f;
  }

  // s += y with the running compensation c (Kahan 1965); finish() adds s - c in double.
  static __device__ __forceinline__ void kahan(float& s, float& c, float y) {
    const float yc = __fsub_rn(y, c);
    const float t = __fadd_rn(s, yc);
    c = __fsub_rn(__fsub_rn(t, s), yc);
    s = t;
  }

  // The neighbour's records, loaded ahead of its pair terms.
  struct Pre {
    float4 xh, xl, vh, vl, q, a;
    float db;
  };
  static constexpr bool kPrefetch = true;

  __device__ __forceinline__ Pre fetch(uint32_t t, uint32_t) const {
    Pre p;
    p.xh = XH[t];
    p.xl = XL[t];
    p.vh = VH[t];
    p.vl = VL[t];
    if (kMom) {
      p.q = Q[t];
      p.a = A[t];
      p.db = 0.f;
    } else {
      p.db = DBp[t];
    }
    return p;
  }

  __device__ __forceinline__ void pair(uint32_t t) { pair_with(t, 0, fetch(t, 0)); }

  __device__ __forceinline__ void pair_with(uint32_t t, uint32_t, const Pre& p) {
    const float4 xj = p.xh, xj2 = p.xl;
    float d[3];
    d[0] = (xh[0] - xj.x) + (xl[0] - xj2.x);
    d[1] = (xh[1] - xj.y) + (xl[1] - xj2.y);
    d[2] = DIM == 3 ? (xh[2] - xj.z) + (xl[2] - xj2.z) : 0.f;
    float r2 = d[0] * d[0] + d[1] * d[1];
    if (DIM == 3) r2 += d[2] * d[2];
    // at r = 2h the spline's F and dF/dr vanish, so an FP32 cut-off there adds nothing
    if (!(r2 < four_h2) || !(r2 > 0.f)) return;
    const float4 vj = p.vh, vj2 = p.vl;
    const float mj = xj.w;
    float inv_r = rsqrtf(r2);
    inv_r = inv_r * fmaf(-0.5f * r2 * inv_r, inv_r, 1.5f);  // one Newton step
    const float r = r2 * inv_r;
    const float q = r * inv_h;
    float F, G;
    if (q < 1.f) {
      F = fa * (2.25f * q - 3.f);
      G = fa * 2.25f * inv_h * inv_r;
    } else {
      const float tq = 2.f - q;
      F = fb * tq * tq * inv_r;
      G = -(fb * tq * inv_r) * (2.f * inv_h + tq * inv_r) * inv_r;
    }
    float dv[3];
    dv[0] = (vh[0] - vj.x) + (vl[0] - vj2.x);
    dv[1] = (vh[1] - vj.y) + (vl[1] - vj2.y);
    dv[2] = DIM == 3 ? (vh[2] - vj.z) + (vl[2] - vj2.z) : 0.f;
    float w = dv[0] * d[0] + dv[1] * d[1];
    if (DIM == 3) w += dv[2] * d[2];
    if (!kMom) {
      const float D = dbi * mj + p.db * mi;
      const float gw = G * w * D, fd = F * D;
#pragma unroll
      for (int c = 0; c < DIM; ++c) {
        kahan(gx[c], cx[c], gw * d[c] + fd * dv[c]);
        kahan(gv[c], cv[c], fd * d[c]);
      }
      return;
    }
    const float4 qj = p.q, aj = p.a;
    const float rb = rhoi + vj.w;
    const float e = r2 + eps_h2;
    float c1 = 0.f, c1a = 0.f;
    // The viscosity acts where the pair approaches (w < 0).  The forward pass decided that on
    // its double-word w; the FP32 w here can carry the wrong sign when |w| is within its rounding
    // of zero (about 4e-7 of sum |dv_c d_c|), and the derivative of the viscosity jumps there, so
    // those rare pairs decide in double (approaches_f64, out of line).
    bool approach = w < 0.f;
    {
      float wabs = fabsf(dv[0] * d[0]) + fabsf(dv[1] * d[1]);
      if (DIM == 3) wabs += fabsf(dv[2] * d[2]);
      if (fabsf(w) <= 1e-5f * wabs) approach = approaches_f64<DIM>(XH, XL, VH, VL, kself, t);
    }
    if (approach) {
      const float base = 1.f / (e * rb);
      c1 = avk * base;
      c1a = avk_alpha * base;
    }
    const float PI = c1 * w;
    const float S = Pi + qj.x + PI;
    float E[3], xE = 0.f;
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
      E[c] = mj * ai[c] - mi * (c == 0 ? aj.x : c == 1 ? aj.y : aj.z);
      xE += d[c] * E[c];
    }
    const float a1 = -G * S * xE + 2.f * F * xE * PI / e;
    const float b1 = -F * c1 * xE;
    const float fs = F * S;
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
      kahan(gx[c], cx[c], a1 * d[c] + b1 * dv[c] - fs * E[c]);
      kahan(gv[c], cv[c], b1 * d[c]);
    }
    kahan(gr, cr, -F * xE * (Pdi - PI / rb));
    const float half = 0.5f * F * xE;
    kahan(gal, ca, -half * c1a * w);
    kahan(gB, cb, -half * (PBi + qj.z));
  }

  __device__ __forceinline__ void finish(const SphArgs& a, const SphK& K, uint32_t id, uint32_t k) {
    double* lx = (double*)a.lam[0];
    double* lv = (double*)a.lam[1];
    double* lr = (double*)a.lam[2];
    if (!kMom) {
#pragma unroll
      for (int c = 0; c < DIM; ++c) {
        const size_t o = (size_t)id * DIM + c;
        lx[o] += (double)gx[c] - (double)cx[c];
        lv[o] += (double)gv[c] - (double)cv[c];
      }
      return;
    }
    const bool fluid = id < K.fluid_end;
    const double dt = K.d.dt;
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
      const size_t o = (size_t)id * DIM + c;
      const double lxo = lx[o];
      lx[o] = lxo + ((double)gx[c] - (double)cx[c]);
      lv[o] = (fluid ? lv[o] + dt * lxo : lv[o]) + ((double)gv[c] - (double)cv[c]);
    }
    const double lrt = lr[id] + ((double)gr - (double)cr);
    lr[id] = lrt;
    ((float*)a.s[6])[k] = (float)(dt * lrt);
    ((double*)a.lam[3])[id] += (double)gal - (double)ca;
    ((double*)a.lam[4])[id] += (double)gB - (double)cb;
  }
};

}  // namespace

int launch_adjoint_prep(cudaStream_t st, const SphArgs& a, bool fp32) {
  if (a.n == 0) return PG_OK;
  const unsigned b = (a.n + 255) / 256;
  if (fp32) {
    if (a.dim == 2) adjoint_prep_f_kernel<2><<<b, 256, 0, st>>>(a);
    else adjoint_prep_f_kernel<3><<<b, 256, 0, st>>>(a);
  } else {
    if (a.dim == 2) adjoint_prep_kernel<2><<<b, 256, 0, st>>>(a);
    else adjoint_prep_kernel<3><<<b, 256, 0, st>>>(a);
  }
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

typedef void (*AdjKernel)(SphArgs, int);

// The two-sided passes of the mixed-precision adjoint (the FP64 adjoint evaluates each pair once:
// pg_adjoint_sym.cu).
template <int DIM>
AdjKernel adjoint_kernel_dim(int stage) {
  return stage == SPH_MOM ? sph_list_pass_kernel<AdjPairsF<DIM, SPH_MOM>, DIM, false>
                          : sph_list_pass_kernel<AdjPairsF<DIM, SPH_CONT>, DIM, false>;
}

AdjKernel adjoint_kernel(int dim, int stage, bool fp32) {
  if (!fp32) return nullptr;
  return dim == 2 ? adjoint_kernel_dim<2>(stage) : adjoint_kernel_dim<3>(stage);
}

// Prefilter positions (float4 x, y, z) of the list kernel and of overflow walks: the FP64 packs
// keep them in s4; the mixed-precision packs use the FP32 hi parts in s0.
int adjoint_pf_index(bool fp32) { return fp32 ? 0 : 4; }

int launch_adjoint_pass(cudaStream_t st, const SphArgs& a, int stage, int grid, bool fp32) {
  if (!fp32) {
    set_error("the FP64 adjoint runs the pair-once kernels");
    return PG_EINVAL;
  }
  if (a.n == 0) return PG_OK;
  const uint32_t ntiles = (a.n + kSphThreads - 1) / kSphThreads;
  if (grid <= 0 || (uint32_t)grid > ntiles) grid = (int)ntiles;
  adjoint_kernel(a.dim, stage, fp32)<<<grid, kSphThreads, 0, st>>>(a, adjoint_pf_index(fp32));
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

int adjoint_pass_occupancy(int dim, int stage, bool fp32) {
  AdjKernel kern = adjoint_kernel(dim, stage, fp32);
  int blocks = 0;
  if (!kern) return 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kern, kSphThreads, 0);
  return e == cudaSuccess ? blocks : 0;
}

namespace {

int copy_state_out(pg_system* s, double* dst) {
  const size_t nd = s->n * (size_t)s->dim;
  PG_CUDA_TRY(cudaMemcpyAsync(dst, s->pos.p, 8 * nd, cudaMemcpyDeviceToDevice, s->stream));
  PG_CUDA_TRY(cudaMemcpyAsync(dst + nd, s->vel.p, 8 * nd, cudaMemcpyDeviceToDevice, s->stream));
  PG_CUDA_TRY(cudaMemcpyAsync(dst + 2 * nd, s->rho.p, 8 * s->n, cudaMemcpyDeviceToDevice, s->stream));
  return PG_OK;
}

int copy_state_in(pg_system* s, const double* src) {
  const size_t nd = s->n * (size_t)s->dim;
  PG_CUDA_TRY(cudaMemcpyAsync(s->pos.p, src, 8 * nd, cudaMemcpyDeviceToDevice, s->stream));
  PG_CUDA_TRY(cudaMemcpyAsync(s->vel.p, src + nd, 8 * nd, cudaMemcpyDeviceToDevice, s->stream));
  PG_CUDA_TRY(cudaMemcpyAsync(s->rho.p, src + 2 * nd, 8 * s->n, cudaMemcpyDeviceToDevice, s->stream));
  return PG_OK;
}

int check_differentiable(pg_system* s) {
  if (s->model != PG_MODEL_SPH || s->nsys != 1 || !s->f64) {
    set_error("differentiation needs a single double-precision SPH system");
    return PG_EINVAL;
  }
  return PG_OK;
}

}  // namespace

}  // namespace pg

namespace {

// The double-word recompute of an IEEE handle's backward pass: enter() switches the handle to
// the double-word mode (the same cell multiplier and block size), leave() restores the IEEE
// mode, the momentum block, the particles per warp and a captured graph.  The destructor
// restores the mode after an early error return.
struct RecomputeMode {
  pg_system* s;
  bool active;
  bool switched = false;
  double mult = 1.0;
  int block = 0, mom = 0, lanes = 1;
  bool graph = false;
  RecomputeMode(pg_system* sys, bool act) : s(sys), active(act) {}
  int enter() {
    if (!active) return PG_OK;
    mult = s->cfg.cell_multiplier;
    block = s->block;
    mom = s->block_mom;
    lanes = s->lanes;
    graph = s->graph_enabled;
    s->graph_enabled = false;
    switched = true;
    return pg::retune_sph(s, mult, PG_F64_FAST, block);
  }
  int leave() {
    if (!switched) return PG_OK;
    switched = false;
    PG_TRY(pg::retune_sph(s, mult, PG_F64_NATIVE, block));
    PG_TRY(pg::set_momentum_block(s, mom));
    PG_TRY(pg::set_pass_lanes(s, lanes));
    if (graph) {
      PG_TRY(pg::capture_graphs(s));
      s->graph_enabled = true;
    }
    return PG_OK;
  }
  ~RecomputeMode() {
    if (switched) leave();
  }
};

}  // namespace

extern "C" {

int pg_forward_checkpointed(pg_system* s, int nsteps, int every) {
  pg::clear_error();
  if (!s) {
    pg::set_error("null handle");
    return PG_EINVAL;
  }
  PG_TRY(pg::check_differentiable(s));
  if (nsteps < 0 || every < 1) {
    pg::set_error("need nsteps >= 0 and every >= 1");
    return PG_EINVAL;
  }
  if (!s->adj) s->adj = new pg_adjoint();
  pg_adjoint* A = s->adj;
  A->have_forward = false;
  A->nsteps = nsteps;
  A->every = every;
  A->nseg = (nsteps + every - 1) / every;
  A->state_doubles = s->n * (size_t)(2 * s->dim + 1);
  const size_t sb = 8 * (A->state_doubles ? A->state_doubles : 1);
  PG_TRY(A->ckpt.ensure(sb * (A->nseg ? A->nseg : 1)));
  PG_TRY(A->final_state.ensure(sb));
  for (int seg = 0; seg < A->nseg; ++seg) {
    PG_TRY(pg::copy_state_out(s, A->ckpt.as<double>() + (size_t)seg * A->state_doubles));
    const int steps = std::min(every, nsteps - seg * every);
    for (int t = 0; t < steps; ++t) PG_TRY(pg::enqueue_sph_step(s, false, 1, nullptr));
  }
  PG_TRY(pg::copy_state_out(s, A->final_state.as<double>()));
  PG_TRY(pg::sync_and_check(s));
  s->nbr_valid = false;
  A->have_forward = true;
  return PG_OK;
}

int pg_backward(pg_system* s, const double* dL_dx, double* dL_dalpha, double* dL_dB, double* dL_dv0) {
  pg::clear_error();
  if (!s) {
    pg::set_error("null handle");
    return PG_EINVAL;
  }
  PG_TRY(pg::check_differentiable(s));
  pg_adjoint* A = s->adj;
  if (!A || !A->have_forward) {
    pg::set_error("call pg_forward_checkpointed first");
    return PG_ESTATE;
  }
  if (!dL_dx && s->n) {
    pg::set_error("null dL/dx");
    return PG_EINVAL;
  }
  const size_t n = s->n, nn = n ? n : 1, nd = n * (size_t)s->dim;
  const size_t ncp1 = s->ncells + 1;
  const int every = A->every;
  // fast f64 handles: mixed-precision adjoint pair terms; IEEE handles: FP64
  const bool fp32 = s->arith == pg::ARITH_F64_DF;
  // An IEEE handle recomputes its segments in the double-word mode (FP32 pipe), from the IEEE
  // checkpoints of the forward run: the recompute then hardly competes with the FP64 adjoint
  // sweep that runs beside it.  Over one segment the recomputed states stay within about 1e-12
  // of the IEEE trajectory (the double-word drift bound), far inside the adjoint's accuracy
  // against the dual-number gradient.  The handle's mode and schedule are restored at the end.
  RecomputeMode mode_guard(s, !fp32);
  PG_TRY(mode_guard.enter());
  for (int b = 0; b < 2; ++b) {
    PG_TRY(A->seg_state[b].ensure(8 * A->state_doubles * every + 8));
    PG_TRY(A->seg_rnext[b].ensure(8 * nn * every));
    PG_TRY(A->seg_cell[b].ensure(4 * nn * every));
    PG_TRY(A->seg_id[b].ensure(4 * nn * every));
    PG_TRY(A->seg_start[b].ensure(4 * ncp1 * every));
  }
  const size_t list_entries = ((nn + pg::kListTile - 1) / pg::kListTile) * pg::kListTile * (size_t)s->list_cap;
  PG_TRY(A->nlist.ensure(4 * list_entries));
  PG_TRY(A->nlen.ensure(4 * nn));
  PG_TRY(A->nresume.ensure(8 * nn));
  if (!A->sweep) {
    PG_CUDA_TRY(cudaStreamCreateWithFlags(&A->sweep, cudaStreamNonBlocking));
    for (int b = 0; b < 2; ++b) {
      PG_CUDA_TRY(cudaEventCreateWithFlags(&A->ev_rec[b], cudaEventDisableTiming));
      PG_CUDA_TRY(cudaEventCreateWithFlags(&A->ev_sweep[b], cudaEventDisableTiming));
    }
  }
  PG_TRY(A->lx.ensure(8 * nn * s->dim));
  PG_TRY(A->lv.ensure(8 * nn * s->dim));
  PG_TRY(A->lr.ensure(8 * nn));
  PG_TRY(A->ga.ensure(8 * nn));
  PG_TRY(A->gb.ensure(8 * nn));
  PG_TRY(A->X4.ensure(32 * (nn + pg::kPackPad)));
  PG_TRY(A->V4.ensure(32 * (nn + pg::kPackPad)));
  PG_TRY(A->Q4.ensure(32 * (nn + pg::kPackPad)));
  PG_TRY(A->A4.ensure(32 * (nn + pg::kPackPad)));
  PG_TRY(A->PF.ensure(16 * (nn + pg::kPackPad)));
  PG_TRY(A->DB.ensure(8 * (nn + pg::kPackPad)));
  if (fp32 && (A->pass_grid_fp32 != (int)fp32 || A->pass_grid[pg::SPH_MOM] == 0)) {
    int dev = 0, sms = 0;
    PG_CUDA_TRY(cudaGetDevice(&dev));
    PG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    for (int st = pg::SPH_CONT; st <= pg::SPH_MOM; ++st)
      A->pass_grid[st] = pg::adjoint_pass_occupancy(s->dim, st, fp32) * sms;
    A->pass_grid_fp32 = (int)fp32;
  }
  if (nd) PG_CUDA_TRY(cudaMemcpyAsync(A->lx.p, dL_dx, 8 * nd, cudaMemcpyHostToDevice, s->stream));
  PG_CUDA_TRY(cudaMemsetAsync(A->lv.p, 0, 8 * nn * s->dim, s->stream));
  PG_CUDA_TRY(cudaMemsetAsync(A->lr.p, 0, 8 * nn, s->stream));
  PG_CUDA_TRY(cudaMemsetAsync(A->ga.p, 0, 8 * nn, s->stream));
  PG_CUDA_TRY(cudaMemsetAsync(A->gb.p, 0, 8 * nn, s->stream));

  pg::SphArgs a = pg::sph_args(s, 0, false);
  if (fp32) {  // float4 packs, carved out of the FP64 pack buffers (same byte counts or less)
    a.s[0] = A->X4.p;
    a.s[1] = (char*)A->X4.p + 16 * nn;
    a.s[2] = A->V4.p;
    a.s[3] = (char*)A->V4.p + 16 * nn;
    a.s[4] = A->Q4.p;
    a.s[5] = A->A4.p;
    a.s[6] = A->DB.p;
    a.s[7] = nullptr;
  } else {  // each pair once (pg_adjoint_sym.cu): entry planes and per-slot partial sums
    const size_t entries = ((nn + pg::kListTile - 1) / pg::kListTile) * pg::kListTile * (size_t)s->list_cap;
    PG_TRY(A->EP.ensure(pg::adjoint_sym_entry_bytes() * entries));
    PG_TRY(A->PS.ensure(pg::adjoint_sym_slot_bytes() * nn));
    a.s[0] = A->X4.p;
    a.s[1] = A->V4.p;
    a.s[2] = A->Q4.p;
    a.s[3] = A->A4.p;
    a.s[4] = A->PF.p;
    a.s[5] = A->DB.p;
    a.s[6] = A->PS.p;
    a.s[7] = nullptr;
    a.fcache = A->EP.p;
  }
  a.lam[0] = A->lx.p;
  a.lam[1] = A->lv.p;
  a.lam[2] = A->lr.p;
  a.lam[3] = A->ga.p;
  a.lam[4] = A->gb.p;
  a.nlist = A->nlist.as<uint32_t>();
  a.nlen = A->nlen.as<uint32_t>();
  a.nresume = A->nresume.as<uint32_t>();
  if (fp32) a.fcache = nullptr;

  // Segment seg recomputed into buffer set b on the handle's stream: the steps from the
  // segment's checkpoint, keeping each step's state, rho' and neighbour structure.  It waits
  // for the sweep that last read the set.
  bool pending[2] = {false, false};
  auto recompute = [&](int seg, int b) -> int {
    if (pending[b]) PG_CUDA_TRY(cudaStreamWaitEvent(s->stream, A->ev_sweep[b], 0));
    const int steps = std::min(every, A->nsteps - seg * every);
    PG_TRY(pg::copy_state_in(s, A->ckpt.as<double>() + (size_t)seg * A->state_doubles));
    for (int t = 0; t < steps; ++t) {
      PG_TRY(pg::copy_state_out(s, A->seg_state[b].as<double>() + (size_t)t * A->state_doubles));
      PG_TRY(pg::enqueue_sph_step(s, false, 1, nullptr));
      if (n) {
        PG_CUDA_TRY(cudaMemcpyAsync(A->seg_rnext[b].as<double>() + (size_t)t * n, s->rho.p, 8 * n,
                                    cudaMemcpyDeviceToDevice, s->stream));
        PG_CUDA_TRY(cudaMemcpyAsync(A->seg_cell[b].as<uint32_t>() + (size_t)t * n, s->nw.sorted_cell, 4 * n,
                                    cudaMemcpyDeviceToDevice, s->stream));
        PG_CUDA_TRY(cudaMemcpyAsync(A->seg_id[b].as<uint32_t>() + (size_t)t * n, s->nw.sorted_id, 4 * n,
                                    cudaMemcpyDeviceToDevice, s->stream));
      }
      PG_CUDA_TRY(cudaMemcpyAsync(A->seg_start[b].as<uint32_t>() + (size_t)t * ncp1, s->nw.cell_start.p, 4 * ncp1,
                                  cudaMemcpyDeviceToDevice, s->stream));
    }
    PG_CUDA_TRY(cudaEventRecord(A->ev_rec[b], s->stream));
    return PG_OK;
  };
  // The adjoint swept back through segment seg (buffer set b) on the sweep stream, after its
  // recompute (and, through the stream order of that recompute, after the setup above).  It
  // touches none of the handle's buffers that a recompute writes.
  auto sweep = [&](int seg, int b) -> int {
    cudaStream_t st = A->sweep;
    PG_CUDA_TRY(cudaStreamWaitEvent(st, A->ev_rec[b], 0));
    const int steps = std::min(every, A->nsteps - seg * every);
    for (int t = steps - 1; t >= 0; --t) {
      const double* sv = A->seg_state[b].as<double>() + (size_t)t * A->state_doubles;
      a.pos = (void*)sv;
      a.vel = (void*)(sv + nd);
      a.rho = (void*)(A->seg_rnext[b].as<double>() + (size_t)t * n);
      a.sorted_cell = A->seg_cell[b].as<uint32_t>() + (size_t)t * n;
      a.sorted_id = A->seg_id[b].as<uint32_t>() + (size_t)t * n;
      a.cell_start = A->seg_start[b].as<uint32_t>() + (size_t)t * ncp1;
      PG_TRY(pg::launch_adjoint_prep(st, a, fp32));
      if (fp32) {
        PG_TRY(pg::launch_sph_list_pf(st, a, pg::adjoint_pf_index(fp32), 0, pg::kSphThreads));
        PG_TRY(pg::launch_adjoint_pass(st, a, pg::SPH_MOM, A->pass_grid[pg::SPH_MOM], fp32));
        PG_TRY(pg::launch_adjoint_pass(st, a, pg::SPH_CONT, A->pass_grid[pg::SPH_CONT], fp32));
      } else {
        PG_TRY(pg::launch_sph_list_exact(st, a, pg::adjoint_pf_index(fp32), 0, pg::kSphThreads));
        for (int part = 0; part < 5; ++part) PG_TRY(pg::launch_adjoint_sym(st, a, part));
      }
    }
    PG_CUDA_TRY(cudaEventRecord(A->ev_sweep[b], st));
    pending[b] = true;
    return PG_OK;
  };
  // the recompute of the previous segment runs beside the sweep of this one
  if (A->nseg > 0) PG_TRY(recompute(A->nseg - 1, 0));
  for (int seg = A->nseg - 1; seg >= 0; --seg) {
    const int b = (A->nseg - 1 - seg) & 1;
    if (seg > 0) PG_TRY(recompute(seg - 1, b ^ 1));
    PG_TRY(sweep(seg, b));
  }
  for (int b = 0; b < 2; ++b)
    if (pending[b]) PG_CUDA_TRY(cudaStreamWaitEvent(s->stream, A->ev_sweep[b], 0));
  PG_TRY(pg::copy_state_in(s, A->final_state.as<double>()));
  std::vector<double> ga(n), gb(n);
  if (n) {
    PG_CUDA_TRY(cudaMemcpyAsync(ga.data(), A->ga.p, 8 * n, cudaMemcpyDeviceToHost, s->stream));
    PG_CUDA_TRY(cudaMemcpyAsync(gb.data(), A->gb.p, 8 * n, cudaMemcpyDeviceToHost, s->stream));
    if (dL_dv0) PG_CUDA_TRY(cudaMemcpyAsync(dL_dv0, A->lv.p, 8 * nd, cudaMemcpyDeviceToHost, s->stream));
  }
  PG_TRY(pg::sync_and_check(s));
  s->nbr_valid = false;
  PG_TRY(mode_guard.leave());
  // fixed-order pairwise sums of the per-particle partials
  auto tree_sum = [](std::vector<double>& v) {
    size_t m = v.size();
    if (m == 0) return 0.0;
    while (m > 1) {
      const size_t h = (m + 1) / 2;
      for (size_t i = 0; i + h < m; ++i) v[i] += v[i + h];
      m = h;
    }
    return v[0];
  };
  if (dL_dalpha) *dL_dalpha = tree_sum(ga);
  if (dL_dB) *dL_dB = tree_sum(gb);
  return PG_OK;
}

}  // extern "C"
