// Arithmetic policies for the pair kernels.
//
//   OpsD  IEEE double, one rounding per operation, never contracted (__dadd_rn, ...).  With
//         the oracle's operation order this reproduces the CPU oracle bit for bit.
//   OpsF  the same in IEEE single precision.
//   OpsFF single precision with contraction allowed (fast f32 mode).
//   df    double-word ("double-float") arithmetic on the FP32 pipe: a value is hi + lo with
//         |lo| <= ulp(hi)/2, about 48 significant bits.  GB300 issues FP32 work ~60x faster
//         than FP64, so the f64 fast mode evaluates the pair terms this way.
//
// Double-word algorithms (all from the published literature, implemented here):
//   TwoSum            Knuth, TAOCP vol. 2 (6 operations, error-free)
//   Fast2Sum          Dekker 1971 (3 operations, error-free when |a| >= |b|)
//   TwoProd           with a fused multiply-add (2 operations, error-free)
//   df_add            "SloppyDWPlusDW" (Dekker 1971; Joldes, Muller & Popescu 2017, Alg. 5):
//                     absolute error <= ~2u^2 (|x| + |y|), u = 2^-24, which is what a sum of
//                     pair terms needs (errors relative to the sum of magnitudes)
//   df_mul            "DWTimesDW3" (Joldes, Muller & Popescu 2017, Alg. 12), rel. error <= 4u^2
//   df_mul_f          "DWTimesFP3" (ibid., Alg. 9), rel. error <= 2u^2
//   df_div            one Newton/Karp-Markstein correction of q1 = x.hi * (1/y.hi) using the
//                     double-word remainder x - q1*y (Karp & Markstein 1997)
//   df_rsqrt          one Newton correction of the FP32 reciprocal square root, with the
//                     residual 1 - a*y^2 formed in double-word arithmetic
#pragma once
#include <cuda_runtime.h>

namespace pg {

struct OpsD {
  typedef double R;
  static __device__ __forceinline__ R add(R a, R b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ R sub(R a, R b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ R mul(R a, R b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ R div(R a, R b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ R sqrt(R a) { return __dsqrt_rn(a); }
};

struct OpsF {
  typedef float R;
  static __device__ __forceinline__ R add(R a, R b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ R sub(R a, R b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ R mul(R a, R b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ R div(R a, R b) { return __fdiv_rn(a, b); }
  static __device__ __forceinline__ R sqrt(R a) { return __fsqrt_rn(a); }
};

struct OpsFF {
  typedef float R;
  static __device__ __forceinline__ R add(R a, R b) { return a + b; }
  static __device__ __forceinline__ R sub(R a, R b) { return a - b; }
  static __device__ __forceinline__ R mul(R a, R b) { return a * b; }
  static __device__ __forceinline__ R div(R a, R b) { return a / b; }
  static __device__ __forceinline__ R sqrt(R a) { return sqrtf(a); }
};

// ---------------------------------------------------------------------------------------
// Double-word arithmetic.
// ---------------------------------------------------------------------------------------
struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(float h, float l) {
  df r;
  r.hi = h;
  r.lo = l;
  return r;
}

__host__ __device__ __forceinline__ void df_split(double x, float* hi, float* lo) {
  const float h = (float)x;
  *hi = h;
  *lo = (float)(x - (double)h);
}

__device__ __forceinline__ df df_from_double(double x) {
  const float h = __double2float_rn(x);
  return df_make(h, __double2float_rn(__dsub_rn(x, (double)h)));
}

__device__ __forceinline__ double df_to_double(df a) { return __dadd_rn((double)a.hi, (double)a.lo); }

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df_make(s, e);
}

__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return df_make(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return df_make(p, __fmaf_rn(a, b, -p));
}

__device__ __forceinline__ df df_neg(df a) { return df_make(-a.hi, -a.lo); }

__device__ __forceinline__ df df_add(df x, df y) {
  const df s = two_sum(x.hi, y.hi);
  const float v = __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo));
  return fast_two_sum(s.hi, v);
}

__device__ __forceinline__ df df_sub(df x, df y) { return df_add(x, df_neg(y)); }

__device__ __forceinline__ df df_add_f(df x, float y) {
  const df s = two_sum(x.hi, y);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, x.lo));
}

__device__ __forceinline__ df df_mul(df x, df y) {
  const df c = two_prod(x.hi, y.hi);
  const float tl0 = __fmul_rn(x.lo, y.lo);
  const float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
  const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
  return fast_two_sum(c.hi, __fadd_rn(c.lo, cl2));
}

__device__ __forceinline__ df df_mul_f(df x, float y) {
  const df c = two_prod(x.hi, y);
  return fast_two_sum(c.hi, __fmaf_rn(x.lo, y, c.lo));
}

__device__ __forceinline__ df df_div(df x, df y) {
  const float t = __frcp_rn(y.hi);
  const float q1 = __fmul_rn(x.hi, t);
  const df r = df_sub(x, df_mul_f(y, q1));
  const float q2 = __fmul_rn(r.hi, t);
  return fast_two_sum(q1, q2);
}

// 1/sqrt(a) for a > 0.
__device__ __forceinline__ df df_rsqrt(df a) {
  const float y = rsqrtf(a.hi);
  const df ay2 = df_mul(a, two_prod(y, y));
  const df e = df_add_f(df_neg(ay2), 1.0f);  // 1 - a*y^2, small
  return fast_two_sum(y, __fmul_rn(__fmul_rn(y, e.hi), 0.5f));
}

}  // namespace pg
