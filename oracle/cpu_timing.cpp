// CPU TIMING BUILD of the SPH step (test infrastructure, not product code): the CPU baseline
// that bench.py times on the host cores.  Only bench.py's CPU-baseline legs and tests/ use it.
//
// It computes the step of prestige_oracle.hpp (same method, same neighbour sets, same
// per-particle summation order) organised the way a tuned CPU code would be:
//   * a parallel stable LSD radix sort of the cell keys (per-thread digit histograms) in place
//     of the oracle's serial counting sort;
//   * state gathered into cell-sorted arrays, so neighbour reads walk contiguous slots;
//   * neighbour lists built once per step (one f64 distance test per candidate), which the
//     continuity and momentum passes both walk, instead of two candidate walks;
//   * compiled with floating-point contraction allowed (-ffp-contract=fast), so the compiler
//     may fuse multiply-adds.  Results therefore differ from the parity build in the last bits;
//     tests/test_cpu_timing.py holds them to 1e-10 normwise per step.
// The reference (dineshadepu/prestige) has no executable particle path (its code generator
// returns text, prestige/src/codegen/simple_cpu.rs:3-22), so this restatement of the method
// is the CPU path the GPU library is compared with.
#include <chrono>
#include <cstdio>
#include <omp.h>

#include "prestige_oracle.hpp"

using namespace pgo;

namespace {

struct TimingSpec {  // same layout as orc_sph_spec in oracle_capi.cpp
  double h, rho0, c0, alpha, eps, B, dt, cell_mult;
  double g[3], lo[3], hi[3];
  long long n_fluid;
  int dim, gamma;
};

// Stable LSD radix sort of (key, id) by key over `bits` key bits, 11 bits per pass, with
// per-thread histograms over contiguous chunks (chunk order = id order, so it is stable).
void radix_sort(size_t n, int bits, std::vector<uint32_t>& key, std::vector<uint32_t>& id,
                std::vector<uint32_t>& key2, std::vector<uint32_t>& id2) {
  const int R = 11, B = 1 << R;
  const int T = omp_get_max_threads();
  std::vector<size_t> hist((size_t)T * B);
  for (int shift = 0; shift < bits; shift += R) {
    std::fill(hist.begin(), hist.end(), 0);
#pragma omp parallel num_threads(T)
    {
      const int t = omp_get_thread_num();
      const size_t a = n * t / T, b = n * (t + 1) / T;
      size_t* h = &hist[(size_t)t * B];
      for (size_t i = a; i < b; ++i) ++h[(key[i] >> shift) & (B - 1)];
#pragma omp barrier
#pragma omp single
      {
        size_t run = 0;
        for (int d = 0; d < B; ++d)
          for (int u = 0; u < T; ++u) {
            const size_t c = hist[(size_t)u * B + d];
            hist[(size_t)u * B + d] = run;
            run += c;
          }
      }
      for (size_t i = a; i < b; ++i) {
        const size_t o = h[(key[i] >> shift) & (B - 1)]++;
        key2[o] = key[i];
        id2[o] = id[i];
      }
    }
    key.swap(key2);
    id.swap(id2);
  }
}

template <class T, int DIM>
struct Stepper {
  SphSpec spec;
  SphConst<T> k;
  Grid g;
  size_t n = 0;
  int cap = DIM == 3 ? 128 : 64;
  std::vector<uint32_t> cell, sid, key2, id2, start;
  std::vector<T> xs[DIM], vs[DIM], rs, ms, rn, Pn;
  std::vector<uint32_t> nl;  // neighbour slots, cap per slot
  std::vector<uint32_t> len;

  void sort_and_gather(SphState<T>& s) {
    const T* pos[3] = {s.x[0].data(), s.x[1].data(), DIM == 3 ? s.x[2].data() : s.x[0].data()};
    cell.resize(n);
    hash_cells<T>(g, n, pos, cell.data());
    sid.resize(n);
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) sid[i] = (uint32_t)i;
    key2.resize(n);
    id2.resize(n);
    int bits = 1;
    while (bits < 32 && (g.ncells() >> bits) > 0) ++bits;
    radix_sort(n, bits, cell, sid, key2, id2);  // cell[] is now the sorted cell of each slot
    const uint64_t nc = g.ncells();
    start.resize(nc + 1);
#pragma omp parallel for schedule(static)
    for (long long q = 0; q <= (long long)n; ++q) {  // every cell start written exactly once
      const uint64_t lo = q == 0 ? 0 : (uint64_t)cell[q - 1] + 1;
      const uint64_t hi = q == (long long)n ? nc : (uint64_t)cell[q];
      for (uint64_t c = lo; c <= hi && c <= nc; ++c) start[c] = (uint32_t)q;
    }
    for (int d = 0; d < DIM; ++d) { xs[d].resize(n); vs[d].resize(n); }
    rs.resize(n); ms.resize(n);
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < (long long)n; ++q) {
      const uint32_t i = sid[q];
      for (int d = 0; d < DIM; ++d) { xs[d][q] = s.x[d][i]; vs[d][q] = s.v[d][i]; }
      rs[q] = s.rho[i];
      ms[q] = s.m[i];
    }
  }

  // Lists of neighbour slots (0 < r^2 < (2h)^2) in the oracle's candidate order; returns the
  // longest list (a list longer than cap is cut and the lists are rebuilt with a larger cap).
  uint32_t build_lists() {
    nl.resize(n * (size_t)cap);
    len.resize(n);
    const int nx = g.n[0], ny = g.n[1], nz = g.n[2], R = g.reach;
    uint32_t longest = 0;
#pragma omp parallel for schedule(dynamic, 512) reduction(max : longest)
    for (long long q = 0; q < (long long)n; ++q) {
      const uint32_t c = cell[q];
      const int cx = (int)(c % nx), cy = (int)((c / nx) % ny), cz = (int)(c / ((uint64_t)nx * ny));
      T xi[3];
      for (int d = 0; d < DIM; ++d) xi[d] = xs[d][q];
      uint32_t* out = &nl[(size_t)q * cap];
      uint32_t m = 0;
      const uint32_t last = (uint32_t)cap - 1;
      const int zr = DIM == 3 ? R : 0;
      for (int dz = -zr; dz <= zr; ++dz) {
        const int z = cz + dz;
        if (z < 0 || z >= nz) continue;
        for (int dy = -R; dy <= R; ++dy) {
          const int y = cy + dy;
          if (y < 0 || y >= ny) continue;
          const int x0 = std::max(cx - R, 0), x1 = std::min(cx + R, nx - 1);
          const uint64_t row = ((uint64_t)z * ny + y) * nx;
          const uint32_t a = start[row + x0], b = start[row + x1 + 1];
          for (uint32_t t = a; t < b; ++t) {  // branch-free append (a list cut at cap is rebuilt)
            T dd[3];
            for (int d = 0; d < DIM; ++d) dd[d] = xi[d] - xs[d][t];
            const T r2 = dist2<T, DIM>(dd);
            out[m < last ? m : last] = t;
            m += (uint32_t)((r2 < k.four_h2) & (r2 > T(0)));
          }
        }
      }
      len[q] = m;
      longest = std::max(longest, m);
    }
    return longest;
  }

  static inline T kernel_factor(const SphConst<T>& k, T r) {
    const T q = r * k.inv_h;
    if (q < T(1)) return k.fa * (T(2.25) * q - T(3.0));
    const T t = T(2.0) - q;
    return k.fb * (t * t) / r;
  }

  void step(SphState<T>& s) {
    sort_and_gather(s);
    uint32_t longest = build_lists();
    while (longest > (uint32_t)cap) {
      cap = (int)longest + 16;
      longest = build_lists();
    }
    rn.resize(n);
    Pn.resize(n);
    // continuity pass: rho' = rho + dt sum_j m_j (v_ij . x_ij) F_ij, then P(rho')
#pragma omp parallel for schedule(dynamic, 512)
    for (long long q = 0; q < (long long)n; ++q) {
      T xi[3], vi[3];
      for (int d = 0; d < DIM; ++d) { xi[d] = xs[d][q]; vi[d] = vs[d][q]; }
      const uint32_t* lst = &nl[(size_t)q * cap];
      T dr = T(0);
      for (uint32_t e = 0; e < len[q]; ++e) {
        const uint32_t t = lst[e];
        T dd[3], dv[3];
        for (int d = 0; d < DIM; ++d) { dd[d] = xi[d] - xs[d][t]; dv[d] = vi[d] - vs[d][t]; }
        const T r2 = dist2<T, DIM>(dd);
        const T F = kernel_factor(k, std::sqrt(r2));
        T w = dv[0] * dd[0] + dv[1] * dd[1];
        if (DIM == 3) w = w + dv[2] * dd[2];
        dr = dr + ms[t] * (w * F);
      }
      rn[q] = rs[q] + k.dt * dr;
      Pn[q] = tait_pterm(k, rn[q]);
    }
    // momentum pass with the new densities, integrator, write-back in id order
#pragma omp parallel for schedule(dynamic, 512)
    for (long long q = 0; q < (long long)n; ++q) {
      const uint32_t i = sid[q];
      s.rho[i] = rn[q];
      if ((size_t)i >= spec.n_fluid) continue;
      T xi[3], vi[3];
      for (int d = 0; d < DIM; ++d) { xi[d] = xs[d][q]; vi[d] = vs[d][q]; }
      const T rhoi = rn[q], Pi = Pn[q];
      const uint32_t* lst = &nl[(size_t)q * cap];
      T a[3] = {T(0), T(0), T(0)};
      for (uint32_t e = 0; e < len[q]; ++e) {
        const uint32_t t = lst[e];
        T dd[3], dv[3];
        for (int d = 0; d < DIM; ++d) { dd[d] = xi[d] - xs[d][t]; dv[d] = vi[d] - vs[d][t]; }
        const T r2 = dist2<T, DIM>(dd);
        const T F = kernel_factor(k, std::sqrt(r2));
        T w = dv[0] * dd[0] + dv[1] * dd[1];
        if (DIM == 3) w = w + dv[2] * dd[2];
        T pij = T(0);
        if (w < T(0)) pij = k.avk * w / ((r2 + k.eps_h2) * (rhoi + rn[t]));
        const T coef = ms[t] * (((Pi + Pn[t]) + pij) * F);
        for (int d = 0; d < DIM; ++d) a[d] = a[d] - coef * dd[d];
      }
      for (int d = 0; d < DIM; ++d) {
        const T v = vi[d] + k.dt * (a[d] + k.g[d]);
        s.v[d][i] = v;
        s.x[d][i] = xi[d] + k.dt * v;
      }
    }
  }
};

template <class T, int DIM>
double run_sorted(const SphSpec& spec, SphState<T>& s, int nsteps) {
  Stepper<T, DIM> st;
  st.spec = spec;
  st.k = sph_consts<T>(spec, T(spec.alpha), T(spec.B));
  st.g = make_grid(DIM, spec.lo, spec.hi, 2.0 * spec.h, spec.cell_mult);
  st.n = s.n;
  auto t0 = std::chrono::steady_clock::now();
  for (int it = 0; it < nsteps; ++it) st.step(s);
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

template <class T>
double run_t(const TimingSpec* sp, size_t n, void* const* state, int nsteps) {
  SphSpec spec;
  spec.dim = sp->dim; spec.h = sp->h; spec.rho0 = sp->rho0; spec.c0 = sp->c0; spec.alpha = sp->alpha;
  spec.eps = sp->eps; spec.B = sp->B; spec.gamma = sp->gamma; spec.dt = sp->dt;
  spec.n_fluid = (size_t)sp->n_fluid; spec.cell_mult = sp->cell_mult;
  for (int d = 0; d < 3; ++d) { spec.g[d] = sp->g[d]; spec.lo[d] = sp->lo[d]; spec.hi[d] = sp->hi[d]; }
  SphState<T> s;
  s.resize(spec.dim, n);
  T* const* cols = (T* const*)state;
  for (int c = 0; c < spec.dim; ++c) {
    std::memcpy(s.x[c].data(), cols[c], sizeof(T) * n);
    std::memcpy(s.v[c].data(), cols[3 + c], sizeof(T) * n);
  }
  std::memcpy(s.rho.data(), cols[6], sizeof(T) * n);
  std::memcpy(s.m.data(), cols[7], sizeof(T) * n);
  const double sec = spec.dim == 2 ? run_sorted<T, 2>(spec, s, nsteps) : run_sorted<T, 3>(spec, s, nsteps);
  for (int c = 0; c < spec.dim; ++c) {
    std::memcpy(cols[c], s.x[c].data(), sizeof(T) * n);
    std::memcpy(cols[3 + c], s.v[c].data(), sizeof(T) * n);
  }
  std::memcpy(cols[6], s.rho.data(), sizeof(T) * n);
  return sec;
}

}  // namespace

extern "C" int orc_timing_threads(int set) {
  if (set > 0) omp_set_num_threads(set);
  return omp_get_max_threads();
}

// nsteps SPH steps in place (state columns as orc_sph_run); returns the wall time in seconds.
extern "C" double orc_sph_run_timing(const TimingSpec* sp, int f64, long long n, void* const* state, int nsteps) {
  if (f64) return run_t<double>(sp, (size_t)n, state, nsteps);
  return run_t<float>(sp, (size_t)n, state, nsteps);
}
