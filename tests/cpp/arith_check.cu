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
  std::printf("arith_check: %d values, %d split mismatches; %d differences, %d out of bound\n", n, bad, m, bad_sub);
  return bad || bad_sub ? 1 : 0;
}
