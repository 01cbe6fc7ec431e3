// extern "C" face of the CPU oracle, loaded with ctypes by the tests and by bench.py's
// CPU-baseline leg.  Test infrastructure only; never linked into the product library.
// All particle arrays are structure-of-arrays in particle-id order.
#include <chrono>
#include <cstdio>
#include <omp.h>

#include "prestige_oracle.hpp"

using namespace pgo;

extern "C" {
struct orc_sph_spec {
  double h, rho0, c0, alpha, eps, B, dt, cell_mult;
  double g[3], lo[3], hi[3];
  long long n_fluid;
  int dim, gamma;
};

struct orc_dem_spec {
  double kn, e, mu, kt, dt, r_max, cell_mult;
  double g[3], lo[3], hi[3], wall_lo[3], wall_hi[3];
  int capacity, pad;
};
}  // extern "C"

static SphSpec to_spec(const orc_sph_spec* s) {
  SphSpec o;
  o.dim = s->dim; o.h = s->h; o.rho0 = s->rho0; o.c0 = s->c0; o.alpha = s->alpha; o.eps = s->eps;
  o.B = s->B; o.gamma = s->gamma; o.dt = s->dt; o.n_fluid = (size_t)s->n_fluid; o.cell_mult = s->cell_mult;
  for (int d = 0; d < 3; ++d) { o.g[d] = s->g[d]; o.lo[d] = s->lo[d]; o.hi[d] = s->hi[d]; }
  return o;
}

static DemSpec to_dem(const orc_dem_spec* s) {
  DemSpec o;
  o.kn = s->kn; o.e = s->e; o.mu = s->mu; o.kt = s->kt; o.dt = s->dt; o.r_max = s->r_max;
  o.cell_mult = s->cell_mult; o.capacity = s->capacity;
  for (int d = 0; d < 3; ++d) {
    o.g[d] = s->g[d]; o.lo[d] = s->lo[d]; o.hi[d] = s->hi[d];
    o.wall_lo[d] = s->wall_lo[d]; o.wall_hi[d] = s->wall_hi[d];
  }
  return o;
}

extern "C" int orc_num_threads(int set) {
  if (set > 0) omp_set_num_threads(set);
  return omp_get_max_threads();
}

// Grid dimensions for a domain; returns the number of cells.
extern "C" long long orc_grid(int dim, const double* lo, const double* hi, double support, double mult, int* n3, int* reach,
                   double* cell) {
  Grid g = make_grid(dim, lo, hi, support, mult);
  for (int d = 0; d < 3; ++d) n3[d] = g.n[d];
  *reach = g.reach;
  *cell = g.cell;
  return (long long)g.ncells();
}

template <class P>
static void build(CellList& cl, int dim, size_t n, const void* x, const void* y, const void* z, const double* lo,
                  const double* hi, double support, double mult) {
  cl.g = make_grid(dim, lo, hi, support, mult);
  const P* pos[3] = {(const P*)x, (const P*)y, dim == 3 ? (const P*)z : (const P*)x};
  build_cell_list<P>(cl, n, pos);
}

// Cell of each particle (id order), slot order and cell-start table (ncells + 1 entries).
extern "C" int orc_cell_list(int dim, int f64, long long n, const void* x, const void* y, const void* z, const double* lo,
                  const double* hi, double support, double mult, uint32_t* cell, uint32_t* sorted_id,
                  uint32_t* start) {
  CellList cl;
  if (f64) build<double>(cl, dim, (size_t)n, x, y, z, lo, hi, support, mult);
  else build<float>(cl, dim, (size_t)n, x, y, z, lo, hi, support, mult);
  std::memcpy(cell, cl.cell.data(), sizeof(uint32_t) * n);
  std::memcpy(sorted_id, cl.sorted_id.data(), sizeof(uint32_t) * n);
  std::memcpy(start, cl.start.data(), sizeof(uint32_t) * cl.start.size());
  return 0;
}

template <class P>
static void counts_t(int dim, size_t n, const void* x, const void* y, const void* z, const double* lo,
                     const double* hi, double support, double mult, uint32_t* counts) {
  CellList cl;
  build<P>(cl, dim, n, x, y, z, lo, hi, support, mult);
  const P* pos[3] = {(const P*)x, (const P*)y, dim == 3 ? (const P*)z : (const P*)x};
  if (dim == 2) neighbor_counts<P, 2>(cl, n, pos, (P)support, counts);
  else neighbor_counts<P, 3>(cl, n, pos, (P)support, counts);
}

extern "C" int orc_neighbor_counts(int dim, int f64, long long n, const void* x, const void* y, const void* z,
                        const double* lo, const double* hi, double support, double mult, uint32_t* counts) {
  if (f64) counts_t<double>(dim, (size_t)n, x, y, z, lo, hi, support, mult, counts);
  else counts_t<float>(dim, (size_t)n, x, y, z, lo, hi, support, mult, counts);
  return 0;
}

// CSR neighbour lists in the fixed traversal order.  offs has n+1 entries; nbr holds cap ids.
template <class P>
static int list_t(int dim, size_t n, const void* x, const void* y, const void* z, const double* lo,
                  const double* hi, double support, double mult, uint64_t* offs, uint32_t* nbr, uint64_t cap) {
  CellList cl;
  build<P>(cl, dim, n, x, y, z, lo, hi, support, mult);
  const P* pos[3] = {(const P*)x, (const P*)y, dim == 3 ? (const P*)z : (const P*)x};
  std::vector<uint64_t> o;
  std::vector<uint32_t> nb;
  if (dim == 2) neighbor_list<P, 2>(cl, n, pos, (P)support, o, nb);
  else neighbor_list<P, 3>(cl, n, pos, (P)support, o, nb);
  std::memcpy(offs, o.data(), sizeof(uint64_t) * (n + 1));
  if (nb.size() > cap) return 3;
  std::memcpy(nbr, nb.data(), sizeof(uint32_t) * nb.size());
  return 0;
}

extern "C" int orc_neighbor_list(int dim, int f64, long long n, const void* x, const void* y, const void* z,
                      const double* lo, const double* hi, double support, double mult, uint64_t* offs,
                      uint32_t* nbr, uint64_t cap) {
  if (f64) return list_t<double>(dim, (size_t)n, x, y, z, lo, hi, support, mult, offs, nbr, cap);
  return list_t<float>(dim, (size_t)n, x, y, z, lo, hi, support, mult, offs, nbr, cap);
}

// eq1 semantics over the neighbour set: dst[i] += sum_{j in N(i)} src[j].
extern "C" int orc_gather_sum(int dim, int f64, long long n, const void* x, const void* y, const void* z, const double* lo,
                   const double* hi, double support, double mult, const double* src, double* dst) {
  CellList cl;
  if (f64) {
    build<double>(cl, dim, (size_t)n, x, y, z, lo, hi, support, mult);
    const double* pos[3] = {(const double*)x, (const double*)y, dim == 3 ? (const double*)z : (const double*)x};
    if (dim == 2) gather_sum<double, 2>(cl, (size_t)n, pos, support, src, dst);
    else gather_sum<double, 3>(cl, (size_t)n, pos, support, src, dst);
  } else {
    build<float>(cl, dim, (size_t)n, x, y, z, lo, hi, support, mult);
    const float* pos[3] = {(const float*)x, (const float*)y, dim == 3 ? (const float*)z : (const float*)x};
    if (dim == 2) gather_sum<float, 2>(cl, (size_t)n, pos, (float)support, src, dst);
    else gather_sum<float, 3>(cl, (size_t)n, pos, (float)support, src, dst);
  }
  return 0;
}

// state: x[3], v[3], rho, m as separate arrays (z/vz ignored in 2D), updated in place.
template <class T>
static void load_state(SphState<T>& s, int dim, size_t n, T* const* st) {
  s.resize(dim, n);
  for (int c = 0; c < dim; ++c) {
    std::memcpy(s.x[c].data(), st[c], sizeof(T) * n);
    std::memcpy(s.v[c].data(), st[3 + c], sizeof(T) * n);
  }
  std::memcpy(s.rho.data(), st[6], sizeof(T) * n);
  std::memcpy(s.m.data(), st[7], sizeof(T) * n);
}

template <class T>
static void store_state(const SphState<T>& s, int dim, size_t n, T* const* st) {
  for (int c = 0; c < dim; ++c) {
    std::memcpy(st[c], s.x[c].data(), sizeof(T) * n);
    std::memcpy(st[3 + c], s.v[c].data(), sizeof(T) * n);
  }
  std::memcpy(st[6], s.rho.data(), sizeof(T) * n);
}

template <class T>
static void rates_t(const orc_sph_spec* sp, size_t n, void* const* state, void* const* out) {
  SphSpec spec = to_spec(sp);
  SphState<T> s;
  load_state<T>(s, spec.dim, n, (T* const*)state);
  SphConst<T> k = sph_consts<T>(spec, T(spec.alpha), T(spec.B));
  CellList cl;
  cl.g = make_grid(spec.dim, spec.lo, spec.hi, 2.0 * spec.h, spec.cell_mult);
  std::vector<T> acc[3], drho;
  if (spec.dim == 2) sph_rates<T, 2>(spec, k, s, cl, acc, drho);
  else sph_rates<T, 3>(spec, k, s, cl, acc, drho);
  for (int c = 0; c < spec.dim; ++c) std::memcpy(out[c], acc[c].data(), sizeof(T) * n);
  std::memcpy(out[3], drho.data(), sizeof(T) * n);
}

// out[0..2] = acceleration without gravity, out[3] = drho/dt.
extern "C" int orc_sph_rates(const orc_sph_spec* sp, int f64, long long n, void* const* state, void* const* out) {
  if (f64) rates_t<double>(sp, (size_t)n, state, out);
  else rates_t<float>(sp, (size_t)n, state, out);
  return 0;
}

template <class T>
static double run_t(const orc_sph_spec* sp, size_t n, void* const* state, int nsteps) {
  SphSpec spec = to_spec(sp);
  SphState<T> s;
  load_state<T>(s, spec.dim, n, (T* const*)state);
  SphConst<T> k = sph_consts<T>(spec, T(spec.alpha), T(spec.B));
  auto t0 = std::chrono::steady_clock::now();
  if (spec.dim == 2) sph_run<T, 2>(spec, k, s, nsteps);
  else sph_run<T, 3>(spec, k, s, nsteps);
  auto t1 = std::chrono::steady_clock::now();
  store_state<T>(s, spec.dim, n, (T* const*)state);
  return std::chrono::duration<double>(t1 - t0).count();
}

// Runs nsteps SPH steps in place; returns the wall time of the steps in seconds.
extern "C" double orc_sph_run(const orc_sph_spec* sp, int f64, long long n, void* const* state, int nsteps) {
  if (f64) return run_t<double>(sp, (size_t)n, state, nsteps);
  return run_t<float>(sp, (size_t)n, state, nsteps);
}

// Half of sph_step (prestige_oracle.hpp) on a state: stage 0 = the continuity pass, rho' into
// rho; stage 1 = the momentum pass with the densities in rho (as rho') and the update of the
// fluid's v and x.  Positions do not change between the stages, so both build the same cell list.
template <class T, int DIM>
static void stage_dim(const SphSpec& spec, const SphConst<T>& k, SphState<T>& s, int stage) {
  CellList cl;
  cl.g = make_grid(DIM, spec.lo, spec.hi, 2.0 * spec.h, spec.cell_mult);
  const T* pos[3] = {s.x[0].data(), s.x[1].data(), DIM == 3 ? s.x[2].data() : s.x[0].data()};
  build_cell_list<T>(cl, s.n, pos);
  std::vector<T> P(s.n);
  if (stage == 0) {
    std::vector<T> rho_new(s.n);
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)s.n; ++i) {
      T a[3], dr;
      sph_pair_loop<T, DIM, true, false>(cl, s, k, P, (size_t)i, a, dr);
      rho_new[i] = s.rho[i] + k.dt * dr;
    }
    s.rho.swap(rho_new);
    return;
  }
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

template <class T>
static void stage_t(const orc_sph_spec* sp, size_t n, void* const* state, int stage) {
  SphSpec spec = to_spec(sp);
  SphState<T> s;
  load_state<T>(s, spec.dim, n, (T* const*)state);
  SphConst<T> k = sph_consts<T>(spec, T(spec.alpha), T(spec.B));
  if (spec.dim == 2) stage_dim<T, 2>(spec, k, s, stage);
  else stage_dim<T, 3>(spec, k, s, stage);
  store_state<T>(s, spec.dim, n, (T* const*)state);
}

extern "C" int orc_sph_stage(const orc_sph_spec* sp, int f64, long long n, void* const* state, int stage) {
  if (stage != 0 && stage != 1) return 1;
  if (f64) stage_t<double>(sp, (size_t)n, state, stage);
  else stage_t<float>(sp, (size_t)n, state, stage);
  return 0;
}

// Flop census of one SPH step on a double state (not modified), counted on one thread.
// out: particles, candidates, pairs, continuity-loop flops, momentum-loop flops, step flops,
// flops of one candidate test.
extern "C" int orc_sph_flop_census(const orc_sph_spec* sp, long long n, void* const* state, double* out) {
  SphSpec spec = to_spec(sp);
  SphState<double> s;
  load_state<double>(s, spec.dim, (size_t)n, (double* const*)state);
  const int threads = omp_get_max_threads();
  omp_set_num_threads(1);  // the flop counter is per thread
  const SphFlopCensus c = spec.dim == 2 ? sph_flop_census<2>(spec, s) : sph_flop_census<3>(spec, s);
  omp_set_num_threads(threads);
  const double v[7] = {c.particles, c.candidates, c.pairs, c.cont_loops, c.mom_loops, c.step, c.test_flops};
  for (int i = 0; i < 7; ++i) out[i] = v[i];
  return 0;
}

// Forward-mode gradient of L = mean_i |x_i(T) - target_i|^2 over fluid particles after nsteps,
// with respect to alpha, B and the initial velocities along direction u (3 dual components).
// state: double arrays as orc_sph_run (not modified); u: dim arrays; target: dim arrays.
// out[0] = L, out[1] = dL/dalpha, out[2] = dL/dB, out[3] = <dL/dv0, u>.
extern "C" int orc_sph_grad_dual(const orc_sph_spec* sp, long long nn, void* const* state, const double* const* u,
                      const double* const* target, int nsteps, double* out) {
  typedef Dual<3> D;
  SphSpec spec = to_spec(sp);
  const size_t n = (size_t)nn;
  SphState<D> s;
  s.resize(spec.dim, n);
  double* const* st = (double* const*)state;
  for (size_t i = 0; i < n; ++i) {
    for (int c = 0; c < spec.dim; ++c) {
      s.x[c][i] = D(st[c][i]);
      s.v[c][i] = D(st[3 + c][i]);
      s.v[c][i].d[2] = u[c][i];
    }
    s.rho[i] = D(st[6][i]);
    s.m[i] = D(st[7][i]);
  }
  D alpha(spec.alpha), B(spec.B);
  alpha.d[0] = 1.0;
  B.d[1] = 1.0;
  SphConst<D> k = sph_consts<D>(spec, alpha, B);
  if (spec.dim == 2) sph_run<D, 2>(spec, k, s, nsteps);
  else sph_run<D, 3>(spec, k, s, nsteps);
  D L(0.0);
  const size_t nf = spec.n_fluid;
  for (size_t i = 0; i < nf; ++i)
    for (int c = 0; c < spec.dim; ++c) {
      D e = s.x[c][i] - D(target[c][i]);
      L = L + e * e;
    }
  L = L / D((double)nf);
  out[0] = L.v;
  out[1] = L.d[0];
  out[2] = L.d[1];
  out[3] = L.d[2];
  return 0;
}

// DEM: state arrays x[3], v[3], w[3], r, m (double, id order) updated in place;
// hpid (n*cap) and hxi (n*cap*3) carry the tangential history in and out.
// Returns the particle-particle contact count of the last step, or -1 on slot overflow.
extern "C" long long orc_dem_run(const orc_dem_spec* sp, long long nn, double* const* state, uint32_t* hpid, double* hxi,
                      int nsteps, double* seconds) {
  DemSpec spec = to_dem(sp);
  const size_t n = (size_t)nn;
  DemState s;
  s.resize(n, spec.capacity);
  for (int c = 0; c < 3; ++c) {
    std::memcpy(s.x[c].data(), state[c], 8 * n);
    std::memcpy(s.v[c].data(), state[3 + c], 8 * n);
    std::memcpy(s.w[c].data(), state[6 + c], 8 * n);
  }
  std::memcpy(s.r.data(), state[9], 8 * n);
  std::memcpy(s.m.data(), state[10], 8 * n);
  std::memcpy(s.hpid.data(), hpid, 4 * n * spec.capacity);
  std::memcpy(s.hxi.data(), hxi, 8 * n * spec.capacity * 3);
  CellList cl;
  cl.g = make_grid(3, spec.lo, spec.hi, 2.0 * spec.r_max, spec.cell_mult);
  long long contacts = 0;
  bool ovf = false;
  auto t0 = std::chrono::steady_clock::now();
  for (int it = 0; it < nsteps; ++it) {
    bool o = false;
    contacts = dem_step(spec, s, cl, &o);
    ovf = ovf || o;
  }
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  for (int c = 0; c < 3; ++c) {
    std::memcpy(state[c], s.x[c].data(), 8 * n);
    std::memcpy(state[3 + c], s.v[c].data(), 8 * n);
    std::memcpy(state[6 + c], s.w[c].data(), 8 * n);
  }
  std::memcpy(hpid, s.hpid.data(), 4 * n * spec.capacity);
  std::memcpy(hxi, s.hxi.data(), 8 * n * spec.capacity * 3);
  return ovf ? -1 : contacts;
}


