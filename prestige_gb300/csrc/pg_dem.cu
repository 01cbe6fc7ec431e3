// DEM: linear spring-dashpot contacts (Cundall & Strack 1979) with a tangential history
// spring capped by Coulomb friction, and the symplectic Euler integrator, in one pass.
//
// Like the SPH pass this is the reference's pairwise gather (prestige/src/lib.rs:7-12,
// prestige/src/codegen/simple_cpu.rs:7-19) with j restricted to the neighbour cells:
//   contact iff |x_ij|^2 < (r_i + r_j)^2;  n = x_ij/|x_ij|;  delta = r_i + r_j - |x_ij|
//   vr = v_i - v_j - (r_i w_i + r_j w_j) x n;  vn = vr.n;  vt = vr - vn n
//   fn = kn delta - gn vn,  gn = gcoef sqrt(m* kn),  gcoef = -2 ln e / sqrt(pi^2 + ln^2 e)
//   xi = (xi_old - (xi_old.n) n) + vt dt;  ft = -kt xi - gn vt
//   |ft| > mu |fn|:  ft <- mu|fn| ft/|ft|,  xi <- -(ft + gn vt)/kt
//   F_i += fn n + ft;  T_i -= r_i n x ft
// plus the six walls of the box (m* = m_i, no partner spin).  Each particle keeps up to
// `capacity` history entries keyed by partner id (walls 0xFFFFFFF0 + face), in contact order.
// All arithmetic is IEEE double in the oracle's operation order, so results are bit-exact.
// Candidates are tested first in FP32 against a conservative bound (GB300 runs FP64 at 1/64
// of the FP32 rate, and nearly every candidate of a settling packing is rejected); the
// survivors go through the exact f64 test of the oracle, so results stay bit-exact.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pg_internal.cuh"
#include "pg_kernels.cuh"

namespace pg {

namespace {

constexpr uint32_t kNoPartner = 0xFFFFFFFFu;
constexpr uint32_t kWallId = 0xFFFFFFF0u;

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// +-0 and 0 < x < inf, tested on the bit pattern.
__device__ __forceinline__ bool is_zero(double x) { return ((unsigned long long)__double_as_longlong(x) << 1) == 0; }
__device__ __forceinline__ bool positive_finite(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return b != 0 && (b >> 52) < 0x7ffull;  // sign clear, not zero, exponent below inf/NaN
}

__device__ __forceinline__ void cross3(const double* a, const double* b, double* c) {
  c[0] = dsub(dmul(a[1], b[2]), dmul(a[2], b[1]));
  c[1] = dsub(dmul(a[2], b[0]), dmul(a[0], b[2]));
  c[2] = dsub(dmul(a[0], b[1]), dmul(a[1], b[0]));
}

struct Contact {
  double nrm[3], delta, vr[3], meff, ri;
};

// The contact law of one contact: its force term fn n + ft, its torque term r_i (n x ft) and the
// new tangential spring.  The owner of the contact adds them in contact order: F += f, T -= t
// (the operation order of the oracle's accumulation).
__device__ __forceinline__ void contact_terms(const DemK& K, const Contact& ct, const double* xo, double* f, double* t,
                                              double* xn) {
  const double* n = ct.nrm;
  const double vn = dadd(dadd(dmul(ct.vr[0], n[0]), dmul(ct.vr[1], n[1])), dmul(ct.vr[2], n[2]));
  double vt[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) vt[c] = dsub(ct.vr[c], dmul(vn, n[c]));
  const double gn = dmul(K.gcoef, __dsqrt_rn(dmul(ct.meff, K.kn)));
  const double fn = dsub(dmul(K.kn, ct.delta), dmul(gn, vn));
  const double xdn = dadd(dadd(dmul(xo[0], n[0]), dmul(xo[1], n[1])), dmul(xo[2], n[2]));
  double xi[3], ft[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) xi[c] = dadd(dsub(xo[c], dmul(xdn, n[c])), dmul(vt[c], K.dt));
#pragma unroll
  for (int c = 0; c < 3; ++c) ft[c] = dsub(dmul(-K.kt, xi[c]), dmul(gn, vt[c]));
  const double ft2 = dadd(dadd(dmul(ft[0], ft[0]), dmul(ft[1], ft[1])), dmul(ft[2], ft[2]));
  const double lim = dmul(K.mu, fabs(fn));
  if (ft2 > dmul(lim, lim)) {
    const double scale = ddiv(lim, __dsqrt_rn(ft2));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      ft[c] = dmul(ft[c], scale);
      xi[c] = ddiv(-dadd(ft[c], dmul(gn, vt[c])), K.kt);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) f[c] = dadd(dmul(fn, n[c]), ft[c]);
  double nxf[3];
  cross3(n, ft, nxf);
#pragma unroll
  for (int c = 0; c < 3; ++c) t[c] = dmul(ct.ri, nxf[c]);
#pragma unroll
  for (int c = 0; c < 3; ++c) xn[c] = xi[c];
}

// One sphere's state as the contact geometry needs it.
struct DemSelf {
  double x[3], v[3], w[3], r, m;
};

__device__ __forceinline__ DemSelf dem_self(const DemArgs& a, uint32_t k) {
  const double4_32a A = a.sA[k], B = a.sB[k], W = a.sW[k];
  DemSelf me;
  me.x[0] = A.x; me.x[1] = A.y; me.x[2] = A.z; me.r = A.w;
  me.v[0] = B.x; me.v[1] = B.y; me.v[2] = B.z; me.m = B.w;
  me.w[0] = W.x; me.w[1] = W.y; me.w[2] = W.z;
  return me;
}

// Geometry of a collected contact of `me`: code = the partner's sorted slot, or kWallId + face.
// Sets the contact and the history key (the partner's id, or the wall code).
__device__ __forceinline__ void contact_geometry(const DemArgs& a, const DemK& K, const DemSelf& me, uint32_t code,
                                                 Contact& ct, uint32_t& pid) {
  ct.ri = me.r;
  if (code < kWallId) {
    const uint32_t t = code;
    pid = a.sorted_id[t];
    const double4_32a Aj = a.sA[t], Bj = a.sB[t], Wj = a.sW[t];
    const double d[3] = {dsub(me.x[0], Aj.x), dsub(me.x[1], Aj.y), dsub(me.x[2], Aj.z)};
    const double d2 = dadd(dadd(dmul(d[0], d[0]), dmul(d[1], d[1])), dmul(d[2], d[2]));
    const double rs = dadd(me.r, Aj.w);
    const double dist = __dsqrt_rn(d2);
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) ct.nrm[cc] = ddiv(d[cc], dist);
    ct.delta = dsub(rs, dist);
    const double wj[3] = {Wj.x, Wj.y, Wj.z};
    const double vj[3] = {Bj.x, Bj.y, Bj.z};
    double ws[3], cr[3];
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) ws[cc] = dadd(dmul(me.r, me.w[cc]), dmul(Aj.w, wj[cc]));
    cross3(ws, ct.nrm, cr);
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) ct.vr[cc] = dsub(dsub(me.v[cc], vj[cc]), cr[cc]);
    const double mj = Bj.w;
    ct.meff = ddiv(dmul(me.m, mj), dadd(me.m, mj));
  } else {
    const int face = (int)(code - kWallId);
    const int ax = face / 2;
    const bool hi_face = face & 1;
    const double dist = hi_face ? dsub(K.wall_hi[ax], me.x[ax]) : dsub(me.x[ax], K.wall_lo[ax]);
    pid = code;
    ct.nrm[0] = ct.nrm[1] = ct.nrm[2] = 0.0;
    ct.nrm[ax] = hi_face ? -1.0 : 1.0;
    ct.delta = dsub(me.r, dist);
    double ws[3], cr[3];
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) ws[cc] = dmul(me.r, me.w[cc]);
    cross3(ws, ct.nrm, cr);
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) ct.vr[cc] = dsub(me.v[cc], cr[cc]);
    ct.meff = me.m;
  }
}

// Tangential spring of partner `pid` in a history row (zero if the pair was not in contact).
__device__ __forceinline__ void history_lookup(const uint32_t* hp, const double* hx, int C, uint32_t pid, double* out) {
  out[0] = out[1] = out[2] = 0.0;
  for (int s = 0; s < C; ++s) {
    const uint32_t q = hp[s];
    if (q == kNoPartner) break;
    if (q == pid) {
      out[0] = hx[s * 3];
      out[1] = hx[s * 3 + 1];
      out[2] = hx[s * 3 + 2];
      break;
    }
  }
}

__global__ void dem_gather_kernel(DemArgs a) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const uint32_t id = a.sorted_id[k];
  const size_t o = (size_t)id * 3;
  a.sA[k] = make_double4_32a(a.pos[o], a.pos[o + 1], a.pos[o + 2], a.radius[id]);
  a.sB[k] = make_double4_32a(a.vel[o], a.vel[o + 1], a.vel[o + 2], a.mass[id]);
  a.sW[k] = make_double4_32a(a.omega[o], a.omega[o + 1], a.omega[o + 2], 0.0);
  a.sF[k] = make_float4((float)a.pos[o], (float)a.pos[o + 1], (float)a.pos[o + 2], (float)a.radius[id]);
}

// The integrator's f64 divisions (a DFMA sequence each on a 1/64-rate pipe), out of line so
// that the particles that skip them (no contact force, no torque) do not run them predicated.
struct D3 {
  double x, y, z;
};

__device__ __noinline__ D3 force_per_mass(D3 F, double m, bool m_ok) {
  D3 r;
  r.x = is_zero(F.x) && m_ok ? F.x : ddiv(F.x, m);
  r.y = is_zero(F.y) && m_ok ? F.y : ddiv(F.y, m);
  r.z = is_zero(F.z) && m_ok ? F.z : ddiv(F.z, m);
  return r;
}

__device__ __noinline__ D3 spin_update(D3 w, D3 T, double I, double dt) {
  D3 r;
  r.x = dadd(w.x, dmul(dt, ddiv(T.x, I)));
  r.y = dadd(w.y, dmul(dt, ddiv(T.y, I)));
  r.z = dadd(w.z, dmul(dt, ddiv(T.z, I)));
  return r;
}

// Contacts a thread collects during its candidate walk before they are evaluated.  The walk
// only tests (FP32 screen, then the exact f64 test).  The contact law then runs for the
// contacts of the whole warp together: the warp's contacts are numbered in (lane, order found)
// order and each lane evaluates one contact of a chunk of 32, whichever particle owns it; each
// owner then adds the terms of its own contacts in the order it found them, so the sums and the
// history are the oracle's, bit for bit.  Evaluated in the walk, each lane's contact ran alone
// while the others waited (a few contacts per particle among about 200 candidates, at different
// iterations per lane); evaluated per lane after the walk, a warp ran as many rounds as its
// busiest lane had contacts.  A lane that collects more than kDemBuf contacts evaluates the
// first kDemBuf itself, in order, before walking on (rare).
constexpr int kDemThreads = 128;
constexpr int kDemWarps = kDemThreads / 32;
constexpr int kDemBuf = 16;

struct DemTerm {  // results of one evaluated contact, for its owner
  double f[3], t[3], xn[3];
  uint32_t pid;
};

__global__ void __launch_bounds__(kDemThreads) dem_pass_kernel(DemArgs a) {
  __shared__ uint32_t s_buf[kDemBuf][kDemThreads];   // [q][thread]: slot of a partner, or kWallId + face
  __shared__ uint16_t s_owner[kDemWarps][32 * kDemBuf];  // warp contact c -> (owner lane << 8) | q
  __shared__ DemTerm s_term[kDemWarps][32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t k = blockIdx.x * blockDim.x + tid;
  const bool live = k < a.n;
  const DemK& K = a.K[0];
  const int C = K.capacity;
  unsigned long long my_contacts = 0;
  const uint32_t id = live ? a.sorted_id[k] : 0u;
  const DemSelf me = dem_self(a, live ? k : 0u);
  uint32_t* hp_new = a.hpid_new + (size_t)id * C;
  double* hx_new = a.hxi_new + (size_t)id * C * 3;
  double F[3] = {0, 0, 0}, T[3] = {0, 0, 0};
  int slot = 0;
  bool overflow = false;
  int nbuf = 0;

  auto store = [&](uint32_t pid, const double* xv) {
    if (slot < C) {
      hp_new[slot] = pid;
      hx_new[slot * 3] = xv[0];
      hx_new[slot * 3 + 1] = xv[1];
      hx_new[slot * 3 + 2] = xv[2];
      ++slot;
    } else {
      overflow = true;
    }
  };
  auto add_terms = [&](const double* f, const double* t) {
#pragma unroll
    for (int c = 0; c < 3; ++c) F[c] = dadd(F[c], f[c]);
#pragma unroll
    for (int c = 0; c < 3; ++c) T[c] = dsub(T[c], t[c]);
  };

  if (live) {
    const uint32_t* hp_old = a.hpid_old + (size_t)id * C;
    const double* hx_old = a.hxi_old + (size_t)id * C * 3;
    // the lane's own evaluation of its buffer (only when it fills during the walk)
    auto flush_own = [&]() {
      for (int q = 0; q < nbuf; ++q) {
        Contact ct;
        uint32_t pid;
        contact_geometry(a, K, me, s_buf[q][tid], ct, pid);
        double xo[3], f[3], t[3], xn[3];
        history_lookup(hp_old, hx_old, C, pid, xo);
        contact_terms(K, ct, xo, f, t, xn);
        add_terms(f, t);
        store(pid, xn);
      }
      nbuf = 0;
    };
    auto collect = [&](uint32_t code) {
      s_buf[nbuf][tid] = code;
      if (++nbuf == kDemBuf) flush_own();
    };

    // FP32 prefilter: |x_i - x_j| < r_i + r_j in f64  =>  the FP32 r^2 below is < thr_j
    // (position and radius rounding to float and the FP32 arithmetic bounded generously)
    const float4 fi = a.sF[k];
    const float Mi = fmaxf(fmaxf(fabsf(fi.x), fabsf(fi.y)), fabsf(fi.z)) + 4.f * fi.w;
    const float slack = 2.384185791015625e-07f * (4.f * Mi) + 1.0e-6f * fi.w;  // 4u (4M) + r rounding

    const GridK& g = K.g;
    const uint32_t c = a.sorted_cell[k] - g.cell_base;
    const int cx = (int)(c % (uint32_t)g.nx);
    const int cy = (int)((c / (uint32_t)g.nx) % (uint32_t)g.ny);
    const int cz = (int)(c / ((uint32_t)g.nx * (uint32_t)g.ny));
    const int R = a.reach;
    const int x0 = max(cx - R, 0), x1 = min(cx + R, g.nx - 1);
    const int side = 2 * R + 1, nrows = side * side;
    // slot range of a row of cells (empty outside the grid); the next row's range is loaded
    // while the current row is walked
    auto row_range = [&](int r, uint32_t& b, uint32_t& e) {
      const int z = cz + r / side - R, y = cy + r % side - R;
      b = e = 0;
      if (z >= 0 && z < g.nz && y >= 0 && y < g.ny) {
        const uint32_t rb = g.cell_base + ((uint32_t)z * g.ny + (uint32_t)y) * g.nx;
        b = a.cell_start[rb + x0];
        e = a.cell_start[rb + x1 + 1];
      }
    };
    uint32_t nb, ne;
    row_range(0, nb, ne);
    for (int row = 0; row < nrows; ++row) {
      const uint32_t s0 = nb, e0 = ne;
      if (row + 1 < nrows) row_range(row + 1, nb, ne);
      for (uint32_t t = s0; t < e0; ++t) {
        {
          const float4 fj = a.sF[t];
          const float d0 = fi.x - fj.x, d1 = fi.y - fj.y, d2 = fi.z - fj.z;
          const float rr = fi.w + fj.w + slack;
          if (!(fmaf(d2, d2, fmaf(d1, d1, d0 * d0)) < rr * rr * 1.0000153f)) continue;
        }
        if (t == k) continue;  // the particle itself (slot k holds id)
        const double4_32a Aj = a.sA[t];
        const double d[3] = {dsub(me.x[0], Aj.x), dsub(me.x[1], Aj.y), dsub(me.x[2], Aj.z)};
        const double d2 = dadd(dadd(dmul(d[0], d[0]), dmul(d[1], d[1])), dmul(d[2], d[2]));
        const double rs = dadd(me.r, Aj.w);
        if (!(d2 < dmul(rs, rs))) continue;
        collect(t);
        ++my_contacts;
      }
    }
    for (int face = 0; face < 6; ++face) {
      const int ax = face / 2;
      const bool hi_face = face & 1;
      // FP32 screen: with every rounding of the FP32 copies bounded (slack), a particle that
      // fails it has dist >= r in f64 as well, so the f64 test is needed only near a wall
      {
        const float xf = ax == 0 ? fi.x : ax == 1 ? fi.y : fi.z;
        const float wf = hi_face ? K.wall_hi_f[ax] : K.wall_lo_f[ax];
        const float df = hi_face ? wf - xf : xf - wf;
        const float wslack = 2.384185791015625e-07f * (2.f * (fabsf(xf) + fabsf(wf)) + fi.w) + 1.0e-6f * fi.w;
        if (df >= fi.w + wslack) continue;
      }
      const double dist = hi_face ? dsub(K.wall_hi[ax], me.x[ax]) : dsub(me.x[ax], K.wall_lo[ax]);
      if (!(dist < me.r)) continue;
      collect(kWallId + (uint32_t)face);
    }
  }

  // ---- the warp's collected contacts, 32 at a time, one per lane (every lane of the warp
  // takes part: lanes without a particle have none) ----
  int first = nbuf;  // exclusive prefix of the lanes' counts = number of the lane's first contact
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, first, off);
    if (lane >= off) first += v;
  }
  const int total = __shfl_sync(0xffffffffu, first, 31);
  first -= nbuf;
  for (int q = 0; q < nbuf; ++q) s_owner[warp][first + q] = (uint16_t)((lane << 8) | q);
  __syncwarp();
  for (int c0 = 0; c0 < total; c0 += 32) {
    const int c = c0 + lane;
    if (c < total) {
      const int own = s_owner[warp][c];
      const int ol = own >> 8, oq = own & 0xff;
      const uint32_t ok = k - (uint32_t)lane + (uint32_t)ol;  // the owner's slot
      const uint32_t oid = a.sorted_id[ok];
      const DemSelf om = dem_self(a, ok);
      Contact ct;
      uint32_t pid;
      contact_geometry(a, K, om, s_buf[oq][warp * 32 + ol], ct, pid);
      double xo[3];
      history_lookup(a.hpid_old + (size_t)oid * C, a.hxi_old + (size_t)oid * C * 3, C, pid, xo);
      DemTerm& r = s_term[warp][lane];
      contact_terms(K, ct, xo, r.f, r.t, r.xn);
      r.pid = pid;
    }
    __syncwarp();
    // each owner adds its contacts of this chunk, in order
    const int lo = max(first, c0), hi = min(first + nbuf, c0 + 32);
    for (int cc = lo; cc < hi; ++cc) {
      const DemTerm& r = s_term[warp][cc - c0];
      add_terms(r.f, r.t);
      store(r.pid, r.xn);
    }
    __syncwarp();
  }

  if (live) {
    // Slots after the last contact must read as empty.  The buffer being written held this
    // particle's history of two steps ago, and every history buffer is empty after its first
    // empty slot (initial state, pg_dem_set_history and this loop keep that), so only the
    // slots up to the old history's end need clearing: usually a single load.
    for (int s = slot; s < C; ++s) {
      if (hp_new[s] == kNoPartner) break;
      hp_new[s] = kNoPartner;
      hx_new[s * 3] = 0.0;
      hx_new[s * 3 + 1] = 0.0;
      hx_new[s * 3 + 2] = 0.0;
    }
    if (overflow) atomicOr(a.err, ERR_CONTACT_OVERFLOW);

    // symplectic Euler: v' = v + dt (F/m + g); x' = x + dt v'; w' = w + dt T / (0.4 m r^2).
    // A particle without contacts has F = T = 0, and 0 / d is that zero (sign kept) for a
    // positive finite d, so those quotients skip the f64 division (1/64-rate pipe on GB300)
    // without changing a bit.
    // The zero and range checks work on the bit patterns (integer pipe).  Without torque and
    // with a finite dt, w' = w + dt * (+-0) is w itself unless w is +-0 (then it is computed).
    const size_t o = (size_t)id * 3;
    const bool free_t = is_zero(T[0]) && is_zero(T[1]) && is_zero(T[2]);
    const double I = free_t ? 0.0 : dmul(dmul(dmul(0.4, me.m), me.r), me.r);
    const bool m_ok = positive_finite(me.m);
    // F / m: the divisions sit behind a branch that the particles without a contact force skip
    // (a select would run them for every particle: the f64 division is a sequence of DFMAs)
    double fm[3] = {F[0], F[1], F[2]};
    if (!(m_ok && is_zero(F[0]) && is_zero(F[1]) && is_zero(F[2]))) {
      const D3 q = force_per_mass(D3{F[0], F[1], F[2]}, me.m, m_ok);
      fm[0] = q.x;
      fm[1] = q.y;
      fm[2] = q.z;
    }
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
      const double v = dadd(me.v[cc], dmul(K.dt, dadd(fm[cc], K.grav[cc])));
      a.vel[o + cc] = v;
      a.pos[o + cc] = dadd(me.x[cc], dmul(K.dt, v));
    }
    if (free_t && K.dt_finite && positive_finite(dmul(dmul(dmul(0.4, me.m), me.r), me.r))) {
#pragma unroll
      for (int cc = 0; cc < 3; ++cc)
        a.omega[o + cc] = is_zero(me.w[cc]) ? dadd(me.w[cc], dmul(K.dt, T[cc])) : me.w[cc];
    } else {
      const D3 w = spin_update(D3{me.w[0], me.w[1], me.w[2]}, D3{T[0], T[1], T[2]}, I, K.dt);
      a.omega[o] = w.x;
      a.omega[o + 1] = w.y;
      a.omega[o + 2] = w.z;
    }
  }
  // contact count: warp sum, one atomic per warp
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) my_contacts += __shfl_down_sync(0xffffffffu, my_contacts, off);
  if ((threadIdx.x & 31) == 0 && my_contacts) atomicAdd(a.contacts, my_contacts);
}

}  // namespace

int launch_dem_gather(cudaStream_t st, const DemArgs& a) {
  if (a.n == 0) return PG_OK;
  dem_gather_kernel<<<(a.n + 255) / 256, 256, 0, st>>>(a);
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

int launch_dem_pass(cudaStream_t st, const DemArgs& a) {
  if (a.n == 0) return PG_OK;
  dem_pass_kernel<<<(a.n + kDemThreads - 1) / kDemThreads, kDemThreads, 0, st>>>(a);
  PG_CUDA_TRY(cudaGetLastError());
  return PG_OK;
}

}  // namespace pg
