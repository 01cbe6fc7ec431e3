// prestige particle hot path -- CPU ORACLE (test infrastructure, not product code).
//
// This header restates, on the CPU, the method that the CUDA library implements:
//   * cell hash, stable (cell, id) ordering, cell-start table          (neighbour search)
//   * the eq1-style gather  dst[i] += src[j]  over the neighbour set     (prestige/src/lib.rs:7-12,
//     executed with the i/j gather semantics of prestige/src/codegen/simple_cpu.rs:7-19)
//   * weakly-compressible SPH: continuity, Tait EOS, Monaghan artificial viscosity,
//     cubic-spline kernel, kick-drift integrator
//   * DEM: linear spring-dashpot normal contact, tangential history spring with a Coulomb cap
//   * a dual-number instantiation of the SPH run for gradient checks
//
// PARITY UNPINNED: the reference (dineshadepu/prestige) contains no executable physics, no
// numeric tests and no golden vectors; its only codegen emits an all-pairs loop as text
// (prestige/src/codegen/simple_cpu.rs:3-22).  The arithmetic here follows the published
// methods (Monaghan 1992 SPH + artificial viscosity, Monaghan & Lattanzio 1985 cubic spline,
// Cundall & Strack 1979 DEM) and is pinned by hand-derived known-answer tests instead.
//
// Only tests/, the smoke check and bench.py's CPU-baseline leg may use this code.
// Build with -ffp-contract=off: the operation order below is the definition of the method.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace pgo {

// ----------------------------------------------------------------------------------------
// Scalars: float, double, or a forward-mode dual number.
// ----------------------------------------------------------------------------------------
inline double value(double x) { return x; }
inline double value(float x) { return (double)x; }

template <int K>
struct Dual {
  double v;
  double d[K];
  Dual() : v(0.0) { for (int k = 0; k < K; ++k) d[k] = 0.0; }
  Dual(double x) : v(x) { for (int k = 0; k < K; ++k) d[k] = 0.0; }
};
template <int K> inline double value(const Dual<K>& x) { return x.v; }
template <int K> inline Dual<K> operator+(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r(a.v + b.v); for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k]; return r;
}
template <int K> inline Dual<K> operator-(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r(a.v - b.v); for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k]; return r;
}
template <int K> inline Dual<K> operator-(const Dual<K>& a) {
  Dual<K> r(-a.v); for (int k = 0; k < K; ++k) r.d[k] = -a.d[k]; return r;
}
template <int K> inline Dual<K> operator*(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r(a.v * b.v); for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k]; return r;
}
template <int K> inline Dual<K> operator/(const Dual<K>& a, const Dual<K>& b) {
  Dual<K> r(a.v / b.v);
  const double ib = 1.0 / b.v;
  for (int k = 0; k < K; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
template <int K> inline Dual<K> sqrt(const Dual<K>& a) {
  Dual<K> r(std::sqrt(a.v));
  const double h = 0.5 / r.v;
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * h;
  return r;
}
template <int K> inline Dual<K> fabs(const Dual<K>& a) { return a.v < 0 ? -a : a; }
using std::sqrt;
using std::fabs;

template <class T> inline bool lt(const T& a, const T& b) { return value(a) < value(b); }

// Primitive type of a scalar: the precision in which integer decisions (cell hash,
// neighbour tests) are made.  A dual number decides on its double value.
template <class T> struct Prim { typedef T type; };
template <int K> struct Prim<Dual<K>> { typedef double type; };
inline float prim(float x) { return x; }
inline double prim(double x) { return x; }
template <int K> inline double prim(const Dual<K>& x) { return x.v; }

// A double that counts its arithmetic, for the flop census of a step (sph_flop_census).  Each
// +, -, *, / and sqrt is one flop; negation, comparisons and conversions are free.  The count
// is kept per thread: run counted code on one thread.
inline uint64_t& flop_count() {
  static thread_local uint64_t c = 0;
  return c;
}
struct Counted {
  double v;
  Counted() : v(0.0) {}
  Counted(double x) : v(x) {}
};
inline double value(const Counted& x) { return x.v; }
inline double prim(const Counted& x) { return x.v; }
template <> struct Prim<Counted> { typedef double type; };
inline Counted operator+(const Counted& a, const Counted& b) { ++flop_count(); return Counted(a.v + b.v); }
inline Counted operator-(const Counted& a, const Counted& b) { ++flop_count(); return Counted(a.v - b.v); }
inline Counted operator*(const Counted& a, const Counted& b) { ++flop_count(); return Counted(a.v * b.v); }
inline Counted operator/(const Counted& a, const Counted& b) { ++flop_count(); return Counted(a.v / b.v); }
inline Counted operator-(const Counted& a) { return Counted(-a.v); }
inline Counted sqrt(const Counted& a) { ++flop_count(); return Counted(std::sqrt(a.v)); }
inline Counted fabs(const Counted& a) { return Counted(std::fabs(a.v)); }

// ----------------------------------------------------------------------------------------
// Cell grid.  Cell side s = mult * support * (1 + 2^-20); the tiny inflation keeps every
// pair closer than `support` within `reach` cells of each other after rounding.
// ----------------------------------------------------------------------------------------
struct Grid {
  int dim = 3;
  double lo[3] = {0, 0, 0};
  double cell = 1.0;
  int n[3] = {1, 1, 1};
  int reach = 1;
  uint64_t ncells() const { return (uint64_t)n[0] * n[1] * n[2]; }
};

inline Grid make_grid(int dim, const double lo[3], const double hi[3], double support, double mult) {
  Grid g;
  g.dim = dim;
  g.cell = mult * support * (1.0 + 0x1p-20);
  for (int d = 0; d < 3; ++d) {
    if (d < dim) {
      g.lo[d] = lo[d];
      g.n[d] = std::max(1, (int)std::ceil((hi[d] - lo[d]) / g.cell));
    } else {
      g.lo[d] = 0.0;
      g.n[d] = 1;
    }
  }
  g.reach = (int)std::ceil(support / g.cell);
  return g;
}

// floor((x - lo) * inv) clamped to [0, n-1], evaluated in precision P.
template <class P>
inline int cell_coord(P x, P lo, P inv, int n) {
  P t = (x - lo) * inv;
  if (!(t >= (P)0)) return 0;
  if (t >= (P)n) return n - 1;
  return (int)t;
}

// Cell index of every particle (particle arrays in id order), precision P.
template <class T>
void hash_cells(const Grid& g, size_t n, const T* const* pos, uint32_t* cell) {
  typedef typename Prim<T>::type P;
  P lo[3], inv = (P)(1.0 / g.cell);
  for (int d = 0; d < 3; ++d) lo[d] = (P)g.lo[d];
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)n; ++i) {
    int c[3] = {0, 0, 0};
    for (int d = 0; d < g.dim; ++d) c[d] = cell_coord<P>(prim(pos[d][i]), lo[d], inv, g.n[d]);
    cell[i] = (uint32_t)(((uint64_t)c[2] * g.n[1] + c[1]) * g.n[0] + c[0]);
  }
}

// Stable counting sort by cell over id order => slots ordered by (cell, id).
// sorted_id[k] = id of the particle in slot k; start[c] .. start[c+1] = slots of cell c.
inline void sort_cells(size_t n, uint64_t ncells, const uint32_t* cell, uint32_t* sorted_id, uint32_t* start) {
  std::vector<uint32_t> count(ncells + 1, 0);
  for (size_t i = 0; i < n; ++i) count[cell[i]]++;
  uint32_t run = 0;
  for (uint64_t c = 0; c < ncells; ++c) { start[c] = run; run += count[c]; }
  start[ncells] = run;
  std::vector<uint32_t> cursor(start, start + ncells);
  for (size_t i = 0; i < n; ++i) sorted_id[cursor[cell[i]]++] = (uint32_t)i;
}

struct CellList {
  Grid g;
  std::vector<uint32_t> cell, sorted_id, start;
};

template <class P>
void build_cell_list(CellList& cl, size_t n, const P* const* pos) {
  cl.cell.resize(n);
  cl.sorted_id.resize(n);
  cl.start.resize(cl.g.ncells() + 1);
  hash_cells<P>(cl.g, n, pos, cl.cell.data());
  sort_cells(n, cl.g.ncells(), cl.cell.data(), cl.sorted_id.data(), cl.start.data());
}

// Visit the candidate partners of a particle in cell `c`, in the fixed order:
// cell rows z, then y (ascending), and along each row the x-cells and their slots ascending.
template <class Fn>
inline void for_each_candidate(const CellList& cl, uint32_t c, Fn&& fn) {
  const Grid& g = cl.g;
  const int nx = g.n[0], ny = g.n[1], nz = g.n[2];
  const int cx = (int)(c % nx);
  const int cy = (int)((c / nx) % ny);
  const int cz = (int)(c / ((uint64_t)nx * ny));
  const int R = g.reach;
  const int zr = g.dim == 3 ? R : 0;
  for (int dz = -zr; dz <= zr; ++dz) {
    const int z = cz + dz;
    if (z < 0 || z >= nz) continue;
    for (int dy = -R; dy <= R; ++dy) {
      const int y = cy + dy;
      if (y < 0 || y >= ny) continue;
      const int x0 = std::max(cx - R, 0), x1 = std::min(cx + R, nx - 1);
      const uint64_t row = ((uint64_t)z * ny + y) * nx;
      const uint32_t s = cl.start[row + x0], e = cl.start[row + x1 + 1];
      for (uint32_t t = s; t < e; ++t) fn(cl.sorted_id[t]);
    }
  }
}

// r^2 in the fixed order dx*dx + dy*dy (+ dz*dz).
template <class T, int DIM>
inline T dist2(const T* d) {
  T r2 = d[0] * d[0] + d[1] * d[1];
  if (DIM == 3) r2 = r2 + d[2] * d[2];
  return r2;
}

// ----------------------------------------------------------------------------------------
// Neighbour lists and the eq1 gather (prestige/src/lib.rs:7-12: force[i] += mass[j]).
// The neighbour set of i is every j (i included) with r_ij^2 < support^2.
// ----------------------------------------------------------------------------------------
template <class P, int DIM>
void neighbor_counts(const CellList& cl, size_t n, const P* const* pos, P support, uint32_t* counts) {
  const P s2 = support * support;
#pragma omp parallel for schedule(dynamic, 256)
  for (long long i = 0; i < (long long)n; ++i) {
    uint32_t cnt = 0;
    for_each_candidate(cl, cl.cell[i], [&](uint32_t j) {
      P d[3];
      for (int k = 0; k < DIM; ++k) d[k] = pos[k][i] - pos[k][j];
      if (dist2<P, DIM>(d) < s2) ++cnt;
    });
    counts[i] = cnt;
  }
}

template <class P, int DIM>
void neighbor_list(const CellList& cl, size_t n, const P* const* pos, P support, std::vector<uint64_t>& offs,
                   std::vector<uint32_t>& nbr) {
  std::vector<uint32_t> counts(n);
  neighbor_counts<P, DIM>(cl, n, pos, support, counts.data());
  offs.assign(n + 1, 0);
  for (size_t i = 0; i < n; ++i) offs[i + 1] = offs[i] + counts[i];
  nbr.resize(offs[n]);
  const P s2 = support * support;
#pragma omp parallel for schedule(dynamic, 256)
  for (long long i = 0; i < (long long)n; ++i) {
    uint64_t o = offs[i];
    for_each_candidate(cl, cl.cell[i], [&](uint32_t j) {
      P d[3];
      for (int k = 0; k < DIM; ++k) d[k] = pos[k][i] - pos[k][j];
      if (dist2<P, DIM>(d) < s2) nbr[o++] = j;
    });
  }
}

template <class P, int DIM>
void gather_sum(const CellList& cl, size_t n, const P* const* pos, P support, const double* src, double* dst) {
  const P s2 = support * support;
#pragma omp parallel for schedule(dynamic, 256)
  for (long long i = 0; i < (long long)n; ++i) {
    double acc = dst[i];
    for_each_candidate(cl, cl.cell[i], [&](uint32_t j) {
      P d[3];
      for (int k = 0; k < DIM; ++k) d[k] = pos[k][i] - pos[k][j];
      if (dist2<P, DIM>(d) < s2) acc = acc + src[j];
    });
    dst[i] = acc;
  }
}

// ----------------------------------------------------------------------------------------
// SPH (weakly compressible).  Cubic spline with support 2h:
//   W(q) = sigma * {1 - 1.5 q^2 + 0.75 q^3 (q<1); 0.25 (2-q)^3 (1<=q<2)},
//   sigma = 10/(7 pi h^2) in 2D, 1/(pi h^3) in 3D.
// grad_i W_ij = F(r) * x_ij with F = (dW/dr)/r:
//   q < 1 : F = fa * (2.25 q - 3),            fa = sigma / h^2
//   q >= 1: F = fb * (2 - q)^2 / r,           fb = -0.75 sigma / h
// Continuity:  drho_i = sum_j m_j (v_ij . x_ij) F_ij
// Momentum:    a_i = -sum_j m_j (P_i + P_j + Pi_ij) F_ij x_ij + g,   P = p / rho^2
// Tait:        p = B ((rho/rho0)^gamma - 1)
// Artificial viscosity (Monaghan 1992) with c_ij = c0, rho_ij = (rho_i + rho_j)/2:
//   Pi_ij = -alpha c0 mu_ij / rho_ij,  mu_ij = h v_ij.x_ij / (r^2 + eps h^2)   if v_ij.x_ij < 0
//         = avk * w / ((r^2 + eps h^2) (rho_i + rho_j)),  avk = -2 alpha c0 h.
// Time step (sph_step): rho' = rho + dt drho(x, v); v' = v + dt (a(x, v, rho') + g); x' = x + dt v'.
// Particles with id >= n_fluid are fixed dummy-wall particles: x, v fixed, rho evolves.
// ----------------------------------------------------------------------------------------
struct SphSpec {
  int dim = 3;
  double h = 0.013, rho0 = 1000.0, c0 = 10.0, alpha = 0.1, eps = 0.01, B = 0.0;
  int gamma = 7;
  double g[3] = {0, 0, 0};
  double dt = 1e-4;
  size_t n_fluid = 0;
  double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  double cell_mult = 1.0;
};

template <class T>
struct SphConst {
  T inv_h, four_h2, fa, fb, avk, eps_h2, B, inv_rho0, dt, g[3];
  int gamma;
};

inline void sph_kernel_factors(int dim, double h, double& fa, double& fb) {
  const double pi = 3.14159265358979323846;
  const double sigma = dim == 2 ? 10.0 / (7.0 * pi * h * h) : 1.0 / (pi * h * h * h);
  fa = sigma / (h * h);
  fb = -0.75 * sigma / h;
}

// alpha and B are passed as T so that a dual-number run can carry their derivatives.
template <class T>
SphConst<T> sph_consts(const SphSpec& s, T alpha, T B) {
  SphConst<T> k;
  double fa, fb;
  sph_kernel_factors(s.dim, s.h, fa, fb);
  k.inv_h = T(1.0 / s.h);
  k.four_h2 = T((2.0 * s.h) * (2.0 * s.h));
  k.fa = T(fa);
  k.fb = T(fb);
  k.avk = T(-2.0 * s.c0 * s.h) * alpha;
  k.eps_h2 = T(s.eps * s.h * s.h);
  k.B = B;
  k.inv_rho0 = T(1.0 / s.rho0);
  k.dt = T(s.dt);
  for (int d = 0; d < 3; ++d) k.g[d] = T(s.g[d]);
  k.gamma = s.gamma;
  return k;
}

template <class T>
inline T tait_pterm(const SphConst<T>& k, T rho) {
  T rr = rho * k.inv_rho0;
  T pw = rr;
  for (int e = 1; e < k.gamma; ++e) pw = pw * rr;
  T p = k.B * (pw - T(1.0));
  return p / (rho * rho);
}

template <class T>
struct SphState {
  int dim = 3;
  size_t n = 0;
  std::vector<T> x[3], v[3], rho, m;
  void resize(int d, size_t nn) {
    dim = d; n = nn;
    for (int k = 0; k < 3; ++k) { x[k].assign(nn, T(0.0)); v[k].assign(nn, T(0.0)); }
    rho.assign(nn, T(0.0)); m.assign(nn, T(0.0));
  }
};

// Pair loop for particle i in the order of for_each_candidate.  CONT accumulates the
// continuity rate, MOM the momentum rate; both share the neighbour test and kernel factor.
template <class T, int DIM, bool CONT, bool MOM>
inline void sph_pair_loop(const CellList& cl, const SphState<T>& s, const SphConst<T>& k, const std::vector<T>& P,
                          size_t i, T* acc, T& drho) {
  T a[3] = {T(0.0), T(0.0), T(0.0)};
  T dr = T(0.0);
  const T xi[3] = {s.x[0][i], s.x[1][i], DIM == 3 ? s.x[2][i] : T(0.0)};
  const T vi[3] = {s.v[0][i], s.v[1][i], DIM == 3 ? s.v[2][i] : T(0.0)};
  const T rhoi = s.rho[i];
  const T Pi = MOM ? P[i] : T(0.0);
  for_each_candidate(cl, cl.cell[i], [&](uint32_t j) {
    T d[3];
    for (int c = 0; c < DIM; ++c) d[c] = xi[c] - s.x[c][j];
    const T r2 = dist2<T, DIM>(d);
    if (!lt(r2, k.four_h2)) return;
    if (!(value(r2) > 0.0)) return;
    const T r = sqrt(r2);
    const T q = r * k.inv_h;
    T F;
    if (value(q) < 1.0) {
      F = k.fa * (T(2.25) * q - T(3.0));
    } else {
      const T t = T(2.0) - q;
      F = k.fb * (t * t) / r;
    }
    T dv[3];
    for (int c = 0; c < DIM; ++c) dv[c] = vi[c] - s.v[c][j];
    T w = dv[0] * d[0] + dv[1] * d[1];
    if (DIM == 3) w = w + dv[2] * d[2];
    const T mj = s.m[j];
    if (CONT) dr = dr + mj * (w * F);
    if (MOM) {
      T pij = T(0.0);
      if (value(w) < 0.0) pij = k.avk * w / ((r2 + k.eps_h2) * (rhoi + s.rho[j]));
      const T coef = mj * (((Pi + P[j]) + pij) * F);
      for (int c = 0; c < DIM; ++c) a[c] = a[c] - coef * d[c];
    }
  });
  for (int c = 0; c < 3; ++c) acc[c] = a[c];
  drho = dr;
}

// SPH rates (acc without gravity, drho) of one state, all particles, arrays in id order.
template <class T, int DIM>
void sph_rates(const SphSpec& spec, const SphConst<T>& k, const SphState<T>& s, CellList& cl, std::vector<T>* acc,
               std::vector<T>& drho) {
  const T* pos[3] = {s.x[0].data(), s.x[1].data(), DIM == 3 ? s.x[2].data() : s.x[0].data()};
  build_cell_list<T>(cl, s.n, pos);
  std::vector<T> P(s.n);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)s.n; ++i) P[i] = tait_pterm(k, s.rho[i]);
  for (int c = 0; c < 3; ++c) acc[c].assign(s.n, T(0.0));
  drho.assign(s.n, T(0.0));
#pragma omp parallel for schedule(dynamic, 256)
  for (long long i = 0; i < (long long)s.n; ++i) {
    T a[3], dr;
    sph_pair_loop<T, DIM, true, true>(cl, s, k, P, (size_t)i, a, dr);
    for (int c = 0; c < 3; ++c) acc[c][i] = a[c];
    drho[i] = dr;
  }
  (void)spec;
}

// One time step: symplectic Euler with the density advanced first.
//   rho' = rho + dt C(x, v)                 C: continuity rate (all particles)
//   v'   = v + dt (M(x, v, rho') + g)       M: momentum rate with the new densities (fluid)
//   x'   = x + dt v'                        (fluid; wall particles keep x and v)
// The acoustic pair (rho, v) is then advanced symplectically (stable for omega dt < 2); a
// single evaluation of both rates from (x, v, rho) would advance it by forward Euler, which
// amplifies every acoustic mode.
template <class T, int DIM>
void sph_step(const SphSpec& spec, const SphConst<T>& k, SphState<T>& s, CellList& cl, std::vector<T>& P) {
  const T* pos[3] = {s.x[0].data(), s.x[1].data(), DIM == 3 ? s.x[2].data() : s.x[0].data()};
  build_cell_list<T>(cl, s.n, pos);
  P.resize(s.n);
  std::vector<T> rho_new(s.n);
#pragma omp parallel for schedule(dynamic, 256)
  for (long long i = 0; i < (long long)s.n; ++i) {
    T a[3], dr;
    sph_pair_loop<T, DIM, true, false>(cl, s, k, P, (size_t)i, a, dr);
    rho_new[i] = s.rho[i] + k.dt * dr;
  }
  s.rho.swap(rho_new);
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)s.n; ++i) P[i] = tait_pterm(k, s.rho[i]);
  std::vector<T> acc[3];
  for (int c = 0; c < DIM; ++c) acc[c].resize(s.n);
#pragma omp parallel for schedule(dynamic, 256)
  for (long long i = 0; i < (long long)s.n; ++i) {
    T a[3], dr;
    sph_pair_loop<T, DIM, false, true>(cl, s, k, P, (size_t)i, a, dr);
    for (int c = 0; c < DIM; ++c) acc[c][i] = a[c];
  }
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)s.n; ++i) {
    if ((size_t)i < spec.n_fluid) {
      for (int c = 0; c < DIM; ++c) {
        s.v[c][i] = s.v[c][i] + k.dt * (acc[c][i] + k.g[c]);
        s.x[c][i] = s.x[c][i] + k.dt * s.v[c][i];
      }
    }
  }
}

template <class T, int DIM>
void sph_run(const SphSpec& spec, const SphConst<T>& k, SphState<T>& s, int nsteps) {
  CellList cl;
  cl.g = make_grid(DIM, spec.lo, spec.hi, 2.0 * spec.h, spec.cell_mult);
  std::vector<T> P;
  for (int it = 0; it < nsteps; ++it) sph_step<T, DIM>(spec, k, s, cl, P);
}

// Flop census of one SPH step (sph_step) on a state, counted with the Counted scalar on the
// calling thread (run it with one OpenMP thread).  The pair loops are counted per particle, so
// their totals split into candidate tests (d and r^2 of a candidate that is not a neighbour,
// the particle itself included) and the pair terms of the neighbours (j != i within 2h).
struct SphFlopCensus {
  double particles = 0, candidates = 0, pairs = 0;
  double cont_loops = 0, mom_loops = 0;  // flops of all continuity / momentum pair loops
  double step = 0;                       // flops of the whole step (loops, Tait, updates)
  double test_flops = 0;                 // flops of one candidate test (d and r^2)
};

template <int DIM>
SphFlopCensus sph_flop_census(const SphSpec& spec, const SphState<double>& s0) {
  SphState<Counted> s;
  s.resize(s0.dim, s0.n);
  for (size_t i = 0; i < s0.n; ++i) {
    for (int c = 0; c < 3; ++c) { s.x[c][i] = s0.x[c][i]; s.v[c][i] = s0.v[c][i]; }
    s.rho[i] = s0.rho[i];
    s.m[i] = s0.m[i];
  }
  const SphConst<Counted> k = sph_consts<Counted>(spec, Counted(spec.alpha), Counted(spec.B));
  SphFlopCensus out;
  out.particles = (double)s.n;
  out.test_flops = 3 * DIM - 1;
  CellList cl;
  cl.g = make_grid(DIM, spec.lo, spec.hi, 2.0 * spec.h, spec.cell_mult);
  const Counted* pos[3] = {s.x[0].data(), s.x[1].data(), DIM == 3 ? s.x[2].data() : s.x[0].data()};
  build_cell_list<Counted>(cl, s.n, pos);
  std::vector<Counted> P(s.n);
  for (size_t i = 0; i < s.n; ++i) P[i] = tait_pterm(k, s.rho[i]);
  for (size_t i = 0; i < s.n; ++i) {
    for_each_candidate(cl, cl.cell[i], [&](uint32_t j) {
      double d[3];
      for (int c = 0; c < DIM; ++c) d[c] = s.x[c][i].v - s.x[c][j].v;
      const double r2 = dist2<double, DIM>(d);
      out.candidates += 1;
      if (r2 < k.four_h2.v && r2 > 0.0) out.pairs += 1;
    });
    Counted a[3], dr;
    flop_count() = 0;
    sph_pair_loop<Counted, DIM, true, false>(cl, s, k, P, i, a, dr);
    out.cont_loops += (double)flop_count();
    flop_count() = 0;
    sph_pair_loop<Counted, DIM, false, true>(cl, s, k, P, i, a, dr);
    out.mom_loops += (double)flop_count();
  }
  std::vector<Counted> Pstep;
  flop_count() = 0;
  sph_step<Counted, DIM>(spec, k, s, cl, Pstep);
  out.step = (double)flop_count();
  flop_count() = 0;
  return out;
}

// ----------------------------------------------------------------------------------------
// DEM: linear spring-dashpot (Cundall & Strack 1979), 3D spheres.
//   contact iff |x_ij|^2 < (r_i + r_j)^2;  n = x_ij / |x_ij|;  delta = r_i + r_j - |x_ij|
//   contact-point relative velocity  vr = v_i - v_j - (r_i w_i + r_j w_j) x n
//   normal:     fn = kn delta - gn (vr . n),  gn = gcoef sqrt(m* kn),
//               gcoef = -2 ln e / sqrt(pi^2 + ln^2 e),  m* = m_i m_j / (m_i + m_j)
//   tangential: xi <- xi_old - (xi_old . n) n + vt dt;  ft = -kt xi - gn vt;
//               if |ft| > mu |fn|: ft <- mu |fn| ft/|ft|,  xi <- -(ft + gn vt) / kt
//   force on i: fn n + ft;  torque on i: -r_i n x ft
// Walls are the six faces of an axis-aligned box, same law with m* = m_i and no partner spin.
// Tangential history is kept per particle, keyed by partner id (walls: 0xFFFFFFF0 + face).
// Symplectic Euler: v' = v + dt (F/m + g); x' = x + dt v'; w' = w + dt tau / (0.4 m r^2).
// ----------------------------------------------------------------------------------------
struct DemSpec {
  double kn = 1e5, e = 0.9, mu = 0.3, kt = 1e5 * 2.0 / 7.0;
  double g[3] = {0, 0, -9.81};
  double dt = 1e-6;
  double r_max = 1e-3;
  double lo[3] = {0, 0, 0}, hi[3] = {0.1, 0.1, 0.3};        // grid extent
  double wall_lo[3] = {0, 0, 0}, wall_hi[3] = {0.1, 0.1, 0.3};
  double cell_mult = 1.0;
  int capacity = 16;
};

inline double dem_gcoef(double e) {
  const double pi = 3.14159265358979323846;
  const double le = std::log(e);
  return -2.0 * le / std::sqrt(pi * pi + le * le);
}

struct DemState {
  size_t n = 0;
  std::vector<double> x[3], v[3], w[3], r, m;
  // history: per particle id, up to `capacity` (partner, xi) entries in contact order
  std::vector<uint32_t> hpid;
  std::vector<double> hxi;
  int capacity = 16;
  void resize(size_t nn, int cap) {
    n = nn; capacity = cap;
    for (int k = 0; k < 3; ++k) { x[k].assign(nn, 0.0); v[k].assign(nn, 0.0); w[k].assign(nn, 0.0); }
    r.assign(nn, 0.0); m.assign(nn, 0.0);
    hpid.assign(nn * cap, 0xFFFFFFFFu);
    hxi.assign(nn * cap * 3, 0.0);
  }
};

static const uint32_t kWallId = 0xFFFFFFF0u;

// One contact (particle or wall partner).  Adds force/torque on i, writes the new history.
struct DemContact {
  double nrm[3], delta, vr[3], meff, ri;
};

inline void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

inline void dem_contact_law(const DemSpec& sp, double gcoef, const DemContact& ct, const double* xi_old, double* F,
                            double* T, double* xi_new) {
  const double* n = ct.nrm;
  const double vn = ct.vr[0] * n[0] + ct.vr[1] * n[1] + ct.vr[2] * n[2];
  double vt[3];
  for (int c = 0; c < 3; ++c) vt[c] = ct.vr[c] - vn * n[c];
  const double gn = gcoef * std::sqrt(ct.meff * sp.kn);
  const double fn = sp.kn * ct.delta - gn * vn;
  const double xdn = xi_old[0] * n[0] + xi_old[1] * n[1] + xi_old[2] * n[2];
  double xi[3], ft[3];
  for (int c = 0; c < 3; ++c) xi[c] = (xi_old[c] - xdn * n[c]) + vt[c] * sp.dt;
  for (int c = 0; c < 3; ++c) ft[c] = -sp.kt * xi[c] - gn * vt[c];
  const double ft2 = ft[0] * ft[0] + ft[1] * ft[1] + ft[2] * ft[2];
  const double lim = sp.mu * std::fabs(fn);
  if (ft2 > lim * lim) {
    const double scale = lim / std::sqrt(ft2);
    for (int c = 0; c < 3; ++c) {
      ft[c] = ft[c] * scale;
      xi[c] = -(ft[c] + gn * vt[c]) / sp.kt;
    }
  }
  for (int c = 0; c < 3; ++c) F[c] = F[c] + (fn * n[c] + ft[c]);
  double nxf[3];
  cross3(n, ft, nxf);
  for (int c = 0; c < 3; ++c) T[c] = T[c] - ct.ri * nxf[c];
  for (int c = 0; c < 3; ++c) xi_new[c] = xi[c];
}

// One DEM step on a state in id order.  Returns the number of particle-particle contacts
// (each counted from both sides); sets *overflow if a particle had more than `capacity` contacts.
inline long long dem_step(const DemSpec& sp, DemState& s, CellList& cl, bool* overflow) {
  const size_t n = s.n;
  const int C = s.capacity;
  const double* pos[3] = {s.x[0].data(), s.x[1].data(), s.x[2].data()};
  build_cell_list<double>(cl, n, pos);
  const double gcoef = dem_gcoef(sp.e);
  std::vector<uint32_t> npid(n * C, 0xFFFFFFFFu);
  std::vector<double> nxi(n * C * 3, 0.0);
  std::vector<double> F(n * 3), Tq(n * 3);
  long long ncontacts = 0;
  bool ovf = false;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : ncontacts) reduction(|| : ovf)
  for (long long ii = 0; ii < (long long)n; ++ii) {
    const size_t i = (size_t)ii;
    double f[3] = {0, 0, 0}, tq[3] = {0, 0, 0};
    int slot = 0;
    const double xi[3] = {s.x[0][i], s.x[1][i], s.x[2][i]};
    const double vi[3] = {s.v[0][i], s.v[1][i], s.v[2][i]};
    const double wi[3] = {s.w[0][i], s.w[1][i], s.w[2][i]};
    const double ri = s.r[i], mi = s.m[i];
    auto lookup = [&](uint32_t pid, double* out) {
      out[0] = out[1] = out[2] = 0.0;
      for (int t = 0; t < C; ++t) {
        const uint32_t q = s.hpid[i * C + t];
        if (q == 0xFFFFFFFFu) break;
        if (q == pid) { for (int c = 0; c < 3; ++c) out[c] = s.hxi[(i * C + t) * 3 + c]; break; }
      }
    };
    auto store = [&](uint32_t pid, const double* xv) {
      if (slot < C) {
        npid[i * C + slot] = pid;
        for (int c = 0; c < 3; ++c) nxi[(i * C + slot) * 3 + c] = xv[c];
        ++slot;
      } else {
        ovf = true;
      }
    };
    for_each_candidate(cl, cl.cell[i], [&](uint32_t j) {
      if (j == i) return;
      double d[3];
      for (int c = 0; c < 3; ++c) d[c] = xi[c] - s.x[c][j];
      const double d2 = dist2<double, 3>(d);
      const double rs = ri + s.r[j];
      if (!(d2 < rs * rs)) return;
      DemContact ct;
      const double dist = std::sqrt(d2);
      for (int c = 0; c < 3; ++c) ct.nrm[c] = d[c] / dist;
      ct.delta = rs - dist;
      double ws[3], cr[3];
      for (int c = 0; c < 3; ++c) ws[c] = ri * wi[c] + s.r[j] * s.w[c][j];
      cross3(ws, ct.nrm, cr);
      for (int c = 0; c < 3; ++c) ct.vr[c] = (vi[c] - s.v[c][j]) - cr[c];
      const double mj = s.m[j];
      ct.meff = mi * mj / (mi + mj);
      ct.ri = ri;
      double xo[3], xn[3];
      lookup(j, xo);
      dem_contact_law(sp, gcoef, ct, xo, f, tq, xn);
      store(j, xn);
      ++ncontacts;
    });
    for (int face = 0; face < 6; ++face) {
      const int ax = face / 2;
      const bool hi_face = face & 1;
      const double dist = hi_face ? sp.wall_hi[ax] - xi[ax] : xi[ax] - sp.wall_lo[ax];
      if (!(dist < ri)) continue;
      DemContact ct;
      for (int c = 0; c < 3; ++c) ct.nrm[c] = 0.0;
      ct.nrm[ax] = hi_face ? -1.0 : 1.0;
      ct.delta = ri - dist;
      double ws[3], cr[3];
      for (int c = 0; c < 3; ++c) ws[c] = ri * wi[c];
      cross3(ws, ct.nrm, cr);
      for (int c = 0; c < 3; ++c) ct.vr[c] = vi[c] - cr[c];
      ct.meff = mi;
      ct.ri = ri;
      double xo[3], xn[3];
      lookup(kWallId + (uint32_t)face, xo);
      dem_contact_law(sp, gcoef, ct, xo, f, tq, xn);
      store(kWallId + (uint32_t)face, xn);
    }
    for (int c = 0; c < 3; ++c) { F[i * 3 + c] = f[c]; Tq[i * 3 + c] = tq[c]; }
  }
#pragma omp parallel for schedule(static)
  for (long long ii = 0; ii < (long long)n; ++ii) {
    const size_t i = (size_t)ii;
    const double mi = s.m[i], ri = s.r[i];
    const double I = 0.4 * mi * ri * ri;
    for (int c = 0; c < 3; ++c) {
      s.v[c][i] = s.v[c][i] + sp.dt * (F[i * 3 + c] / mi + sp.g[c]);
      s.x[c][i] = s.x[c][i] + sp.dt * s.v[c][i];
      s.w[c][i] = s.w[c][i] + sp.dt * (Tq[i * 3 + c] / I);
    }
  }
  s.hpid.swap(npid);
  s.hxi.swap(nxi);
  if (overflow) *overflow = ovf;
  return ncontacts;
}

}  // namespace pgo
