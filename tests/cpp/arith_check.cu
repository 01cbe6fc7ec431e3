// Device checks of the double-word helpers in prestige_gb300/csrc/pg_arith.cuh, run by
// tests/test_gpu_arith.py.
//
//   df_split_fast   the integer-only split must give the bits of the hardware conversions
//                   (hi = RN32(x), lo = RN32(x - hi)) for every finite double, zero's sign of lo
//                   aside; checked on random doubles over the whole exponent range and on the
//                   rounding edge cases (ties to even, carries into the exponent, the limits of
//                   the integer path)
//   df_sub_close    exact hi difference: when the hi parts are within a factor 2, hi + lo equals
//                   the difference of the operands to within one rounding of the lo difference
//                   (2^-46 of the operands' magnitude)
//   df_div          quotient of double-word operands within 2^-43 of the f64 quotient of their
//                   values (the approximate-reciprocal seed plus one correction)
//   df_add_raw      the value of df_add (within 2^-46 of |x| + |y|), its lo part at most
//                   2^-23 (|hi| + |x| + |y|)
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <random>
#include <vector>

#include "../../prestige_gb300/csrc/pg_arith.cuh"

using namespace pg;

__global__ void split_kernel(const double* x, int n, float* h1, float* l1, float* h2, float* l2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  df_split(x[i], &h1[i], &l1[i]);
  df_split_fast(x[i], &h2[i], &l2[i]);
}

__global__ void sub_kernel(const double* a, const double* b, int n, double* exact, double* got) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float ah, al, bh, bl;
  df_split(a[i], &ah, &al);
  df_split(b[i], &bh, &bl);
  const df d = df_sub_close(df_make(ah, al), df_make(bh, bl));
  // the f64 value of the double-word difference of the double-words (exact in f64)
  exact[i] = __dsub_rn(__dadd_rn((double)ah, (double)al), __dadd_rn((double)bh, (double)bl));
  got[i] = __dadd_rn((double)d.hi, (double)d.lo);
}

__global__ void div_add_kernel(const double* a, const double* b, int n, double* q, double* sn, double* sr,
                               float* rhi, float* rlo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float ah, al, bh, bl;
  df_split(a[i], &ah, &al);
  df_split(b[i], &bh, &bl);
  const df x = df_make(ah, al), y = df_make(bh, bl);
  const df d = df_div(x, y);
  q[i] = __dadd_rn((double)d.hi, (double)d.lo);
  const df s = df_add(x, y), r = df_add_raw(x, y);
  sn[i] = __dadd_rn((double)s.hi, (double)s.lo);
  sr[i] = __dadd_rn((double)r.hi, (double)r.lo);
  rhi[i] = r.hi;
  rlo[i] = r.lo;
}

static double from_bits(uint64_t b) {
  double x;
  std::memcpy(&x, &b, 8);
  return x;
}

int main() {
  std::mt19937_64 rng(42);
  std::vector<double> xs;
  // random bit patterns (finite only), then values in the integer path's exponent range
  for (int i = 0; i < 200000; ++i) {
    const uint64_t b = rng();
    const double x = from_bits(b);
    if (x == x && x - x == 0.0) xs.push_back(x);
  }
  std::uniform_real_distribution<double> U(-4.0, 4.0);
  for (int i = 0; i < 200000; ++i) xs.push_back(U(rng) * std::ldexp(1.0, (int)(rng() % 200) - 90));
  // rounding edges: ties (rest == 2^28) with even and odd m23, carries into the exponent,
  // and the exponent limits of the integer path
  for (int e = -75; e <= 130; ++e) {
    const uint64_t ebits = (uint64_t)(e + 1023) << 52;
    for (uint64_t m23 : {0ull, 1ull, 2ull, 0x7ffffeull, 0x7fffffull, 0x400000ull}) {
      for (uint64_t rest : {0ull, 1ull, 0xfffffffull, 0x10000000ull, 0x10000001ull, 0x1fffffffull}) {
        const uint64_t b = ebits | (m23 << 29) | rest;
        xs.push_back(from_bits(b));
        xs.push_back(-from_bits(b));
      }
    }
  }
  xs.push_back(0.0);
  xs.push_back(-0.0);
  const int n = (int)xs.size();
  double* dx;
  float *h1, *l1, *h2, *l2;
  cudaMalloc(&dx, 8 * n);
  cudaMalloc(&h1, 4 * n);
  cudaMalloc(&l1, 4 * n);
  cudaMalloc(&h2, 4 * n);
  cudaMalloc(&l2, 4 * n);
  cudaMemcpy(dx, xs.data(), 8 * n, cudaMemcpyHostToDevice);
  split_kernel<<<(n + 255) / 256, 256>>>(dx, n, h1, l1, h2, l2);
  std::vector<float> H1(n), L1(n), H2(n), L2(n);
  cudaMemcpy(H1.data(), h1, 4 * n, cudaMemcpyDeviceToHost);
  cudaMemcpy(L1.data(), l1, 4 * n, cudaMemcpyDeviceToHost);
  cudaMemcpy(H2.data(), h2, 4 * n, cudaMemcpyDeviceToHost);
  cudaMemcpy(L2.data(), l2, 4 * n, cudaMemcpyDeviceToHost);
  if (cudaGetLastError() != cudaSuccess) {
    std::fprintf(stderr, "CUDA error\n");
    return 2;
  }
  int bad = 0;
  for (int i = 0; i < n; ++i) {
    uint32_t a, b, c, d;
    std::memcpy(&a, &H1[i], 4);
    std::memcpy(&b, &H2[i], 4);
    std::memcpy(&c, &L1[i], 4);
    std::memcpy(&d, &L2[i], 4);
    const bool lo_ok = c == d || (L1[i] == 0.f && L2[i] == 0.f);
    if (a != b || !lo_ok) {
      if (bad < 10) std::fprintf(stderr, "split %.17g: hw (%a, %a) fast (%a, %a)\n", xs[i], H1[i], L1[i], H2[i], L2[i]);
      ++bad;
    }
  }
  // df_sub_close on positions shifted to [8h, 8h + extent] (h = 0.013, extent up to 3)
  const int m = 100000;
  std::vector<double> A(m), B(m);
  std::uniform_real_distribution<double> P(0.104, 3.104), D(-0.026, 0.026);
  for (int i = 0; i < m; ++i) {
    A[i] = P(rng);
    B[i] = std::max(0.104, A[i] + D(rng));
  }
  double *da, *db, *de, *dg;
  cudaMalloc(&da, 8 * m);
  cudaMalloc(&db, 8 * m);
  cudaMalloc(&de, 8 * m);
  cudaMalloc(&dg, 8 * m);
  cudaMemcpy(da, A.data(), 8 * m, cudaMemcpyHostToDevice);
  cudaMemcpy(db, B.data(), 8 * m, cudaMemcpyHostToDevice);
  sub_kernel<<<(m + 255) / 256, 256>>>(da, db, m, de, dg);
  std::vector<double> E(m), G(m);
  cudaMemcpy(E.data(), de, 8 * m, cudaMemcpyDeviceToHost);
  cudaMemcpy(G.data(), dg, 8 * m, cudaMemcpyDeviceToHost);
  int bad_sub = 0;
  for (int i = 0; i < m; ++i)
    if (std::fabs(G[i] - E[i]) > std::ldexp(std::max(std::fabs(A[i]), std::fabs(B[i])), -46)) {
      if (bad_sub < 10) std::fprintf(stderr, "sub %.17g - %.17g: %.17g vs %.17g\n", A[i], B[i], G[i], E[i]);
      ++bad_sub;
    }
  // df_div and df_add_raw on operands over 12 decades, both signs
  std::vector<double> X(m), Y(m);
  std::uniform_real_distribution<double> Dec(-6.0, 6.0), S(0.0, 1.0);
  for (int i = 0; i < m; ++i) {
    X[i] = std::pow(10.0, Dec(rng)) * (S(rng) < 0.5 ? -1.0 : 1.0);
    Y[i] = std::pow(10.0, Dec(rng)) * (S(rng) < 0.5 ? -1.0 : 1.0);
  }
  double *dq, *dsn, *dsr;
  float *drh, *drl;
  cudaMalloc(&dq, 8 * m);
  cudaMalloc(&dsn, 8 * m);
  cudaMalloc(&dsr, 8 * m);
  cudaMalloc(&drh, 4 * m);
  cudaMalloc(&drl, 4 * m);
  cudaMemcpy(da, X.data(), 8 * m, cudaMemcpyHostToDevice);
  cudaMemcpy(db, Y.data(), 8 * m, cudaMemcpyHostToDevice);
  div_add_kernel<<<(m + 255) / 256, 256>>>(da, db, m, dq, dsn, dsr, drh, drl);
  std::vector<double> Q(m), SN(m), SR(m);
  std::vector<float> RH(m), RL(m);
  cudaMemcpy(Q.data(), dq, 8 * m, cudaMemcpyDeviceToHost);
  cudaMemcpy(SN.data(), dsn, 8 * m, cudaMemcpyDeviceToHost);
  cudaMemcpy(SR.data(), dsr, 8 * m, cudaMemcpyDeviceToHost);
  cudaMemcpy(RH.data(), drh, 4 * m, cudaMemcpyDeviceToHost);
  cudaMemcpy(RL.data(), drl, 4 * m, cudaMemcpyDeviceToHost);
  if (cudaGetLastError() != cudaSuccess) {
    std::fprintf(stderr, "CUDA error\n");
    return 2;
  }
  int bad_div = 0, bad_add = 0;
  for (int i = 0; i < m; ++i) {
    float xh, xl, yh, yl;
    df_split(X[i], &xh, &xl);
    df_split(Y[i], &yh, &yl);
    const double xv = (double)xh + (double)xl, yv = (double)yh + (double)yl;
    const double qref = xv / yv;
    if (!(std::fabs(Q[i] - qref) <= std::ldexp(std::fabs(qref), -43))) {
      if (bad_div < 10) std::fprintf(stderr, "div %.17g / %.17g: %.17g vs %.17g\n", xv, yv, Q[i], qref);
      ++bad_div;
    }
    const double scale = std::fabs(xv) + std::fabs(yv);
    const bool val_ok = std::fabs(SR[i] - SN[i]) <= std::ldexp(scale, -46);
    const bool lo_ok = std::fabs((double)RL[i]) <= std::ldexp(std::fabs((double)RH[i]) + scale, -23);
    if (!val_ok || !lo_ok) {
      if (bad_add < 10) std::fprintf(stderr, "add_raw %.17g + %.17g: %.17g vs %.17g (lo %a hi %a)\n", xv, yv, SR[i], SN[i], RL[i], RH[i]);
      ++bad_add;
    }
  }
  std::printf("arith_check: %d values, %d split mismatches; %d differences, %d out of bound; %d quotients, %d out of "
              "bound; %d raw sums, %d out of bound\n", n, bad, m, bad_sub, m, bad_div, m, bad_add);
  return bad || bad_sub || bad_div || bad_add ? 1 : 0;
}
