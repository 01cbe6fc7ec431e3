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
//   df_sub_close      x - y for operands whose hi parts are within a factor 2 (Sterbenz)
//   df_add            "SloppyDWPlusDW" (Dekker 1971; Joldes, Muller & Popescu 2017, Alg. 5):
//                     absolute error <= ~2u^2 (|x| + |y|), u = 2^-24, which is what a sum of
//                     pair terms needs (errors relative to the sum of magnitudes)
//   df_mul            "DWTimesDW3" (Joldes, Muller & Popescu 2017, Alg. 12), rel. error <= 4u^2
//   df_mul_f          "DWTimesFP3" (ibid., Alg. 9), rel. error <= 2u^2
//   df_add_raw        df_add without its final Fast2Sum: the same value, with a lo part of up to
//                     about 2^-24 (|x| + |y|), more than ulp(hi)/2 where x and y cancel.  For
//                     operands of products and dot products (df_mul, df_mul_f, df_div, df_dot3,
//                     dfacc_add_prod), which take hi into an error-free transform and lo into an
//                     FP32 correction term: the rounding of that term, 2^-24 |lo| times the other
//                     factor, stays within the sum's own error bound (~2u^2 (|x| + |y|)) times it
//   df_div            one Newton/Karp-Markstein correction of q1 = x.hi * t, t the hardware
//                     approximate reciprocal of y.hi (rcp.approx, relative error below 2^-23), using
//                     the double-word remainder x - q1*y (Karp & Markstein 1997): the correction
//                     leaves a relative error of about t's error squared, below 2^-44
//   df_rsqrt          one Newton correction of the FP32 reciprocal square root, with the
//                     residual 1 - a*y^2 (about 2^-22) formed by FMAs to about 2^-46 absolute
//   df_sumsq3 /       |x|^2 and x.y of 3-vectors: the three hi products by TwoProd, summed by
//   df_dot3           TwoSum, with every second-order term (product errors, hi*lo cross terms,
//                     sum errors) collected in one FP32 correction (about 30 operations in place
//                     of 3 products and 2 sums, ~49); error <= ~4u^2 times the sum of |products|
//   dfacc             an unnormalised accumulator: a += x*y adds the TwoProd hi part by TwoSum
//                     and every lower-order part into acc.lo (12 operations in place of a
//                     product and a sum, ~20); over n terms the error stays below
//                     ~(n^2/2) u^2 max|x*y|, 2e-11 max|x*y| for n = 74
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

// hi = RN32(x), lo = RN32(x - hi) with integer operations only (GB300 issues FP64 and its
// conversions at 1/64 of the FP32 rate).  The binary64 significand is rounded to 24 bits
// (nearest, ties to even) and the exact remainder, an integer of at most 30 bits times
// 2^(e-52), is converted with one integer-to-float rounding and scaled by a power of two.
// Exponents outside [-70, 126], zeros, infinities and NaNs take the hardware conversions.
// The hardware-conversion path, out of line: rare exponents only, so the common path does not
// compute it as well (the f64 conversions run at the 1/64 rate on GB300).
static __device__ __noinline__ float2 df_split_slow(double x) {
  float2 r;
  df_split(x, &r.x, &r.y);
  return r;
}

__device__ __forceinline__ void df_split_fast(double x, float* hi, float* lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if (e < -70 || e > 126) {
    const float2 r = df_split_slow(x);
    *hi = r.x;
    *lo = r.y;
    return;
  }
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const unsigned long long mant = b & 0xfffffffffffffull;
  const unsigned m23 = (unsigned)(mant >> 29);
  const unsigned rest = (unsigned)(mant & 0x1fffffffu);
  const unsigned up = (rest > 0x10000000u || (rest == 0x10000000u && (m23 & 1u))) ? 1u : 0u;
  // hi: carry of the rounding into the exponent is handled by the integer addition
  const unsigned hbits = (((unsigned)(e + 127) << 23) | m23) + up;
  *hi = __uint_as_float(sign | hbits);
  // remainder in units of 2^(e-52): rest - up * 2^29, in [-2^28, 2^28]
  const int r = (int)rest - (int)(up << 29);
  const float scale = __uint_as_float((unsigned)(e - 52 + 127) << 23);
  *lo = __uint_as_float(__float_as_uint(__int2float_rn(r) * scale) ^ sign);
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

__device__ __forceinline__ df df_add_raw(df x, df y) {
  const df s = two_sum(x.hi, y.hi);
  return df_make(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

__device__ __forceinline__ df df_sub_raw(df x, df y) { return df_add_raw(x, df_neg(y)); }

// Approximate reciprocal (PTX rcp.approx.ftz.f32: relative error below 2^-23, subnormals
// flushed); the seed of df_div, whose correction step makes up the difference.
__device__ __forceinline__ float rcp_approx(float y) {
  float t;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(t) : "f"(y));
  return t;
}

// x - y when the hi parts lie within a factor 2 of each other, so that their difference is exact
// (Sterbenz 1974): 5 operations in place of 11.  Fast2Sum applies because a nonzero hi
// difference is at least one ulp of the operands and each lo part is at most half of one.
__device__ __forceinline__ df df_sub_close(df x, df y) {
  return fast_two_sum(__fsub_rn(x.hi, y.hi), __fsub_rn(x.lo, y.lo));
}

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

// y.hi must be a normal float (the divisors here are densities and squared distances).
__device__ __forceinline__ df df_div(df x, df y) {
  const float t = rcp_approx(y.hi);
  const float q1 = __fmul_rn(x.hi, t);
  const df r = df_sub(x, df_mul_f(y, q1));
  const float q2 = __fmul_rn(r.hi, t);
  return fast_two_sum(q1, q2);
}

// 1/sqrt(a) for a > 0.  The residual e = 1 - a y^2 of the FP32 seed y is about 2^-22, so its
// leading bits suffice: a.hi y = h + l exactly (TwoProd), h y - 1 by one FMA (absolute error
// about 2^-46), the small terms l y and a.lo y^2 in FP32.  Then y + y e / 2 (Newton).
__device__ __forceinline__ df df_rsqrt(df a) {
  const float y = rsqrtf(a.hi);
  const float h = __fmul_rn(a.hi, y);
  const float l = __fmaf_rn(a.hi, y, -h);
  const float r = __fmaf_rn(h, y, -1.0f);
  const float e = -__fmaf_rn(__fmaf_rn(a.lo, y, l), y, r);
  return fast_two_sum(y, __fmul_rn(__fmul_rn(y, e), 0.5f));
}

// |a|^2 of the vector (a0, a1, a2); pass a zero for a2 in 2D.
__device__ __forceinline__ df df_sumsq3(df a0, df a1, df a2) {
  const float p0 = __fmul_rn(a0.hi, a0.hi), p1 = __fmul_rn(a1.hi, a1.hi), p2 = __fmul_rn(a2.hi, a2.hi);
  const float e0 = __fmaf_rn(a0.hi, a0.hi, -p0), e1 = __fmaf_rn(a1.hi, a1.hi, -p1);
  const float e2 = __fmaf_rn(a2.hi, a2.hi, -p2);
  float t = a0.hi * a0.lo;
  t = fmaf(a1.hi, a1.lo, t);
  t = fmaf(a2.hi, a2.lo, t);
  const df s1 = two_sum(p0, p1);
  const df s2 = two_sum(s1.hi, p2);
  const float lo = ((e0 + e1) + fmaf(2.f, t, e2)) + (s1.lo + s2.lo);
  return fast_two_sum(s2.hi, lo);
}

// a . b of 3-vectors; pass zeros for the third components in 2D.
__device__ __forceinline__ df df_dot3(df a0, df a1, df a2, df b0, df b1, df b2) {
  const float p0 = __fmul_rn(a0.hi, b0.hi), p1 = __fmul_rn(a1.hi, b1.hi), p2 = __fmul_rn(a2.hi, b2.hi);
  const float e0 = __fmaf_rn(a0.hi, b0.hi, -p0), e1 = __fmaf_rn(a1.hi, b1.hi, -p1);
  const float e2 = __fmaf_rn(a2.hi, b2.hi, -p2);
  float t = a0.hi * b0.lo;
  t = fmaf(a0.lo, b0.hi, t);
  t = fmaf(a1.hi, b1.lo, t);
  t = fmaf(a1.lo, b1.hi, t);
  t = fmaf(a2.hi, b2.lo, t);
  t = fmaf(a2.lo, b2.hi, t);
  const df s1 = two_sum(p0, p1);
  const df s2 = two_sum(s1.hi, p2);
  const float lo = ((e0 + e1) + (e2 + t)) + (s1.lo + s2.lo);
  return fast_two_sum(s2.hi, lo);
}

// Unnormalised double-word accumulator (value hi + lo).
struct dfacc {
  float hi, lo;
};

__device__ __forceinline__ dfacc dfacc_zero() {
  dfacc a;
  a.hi = a.lo = 0.f;
  return a;
}

// a += x * y
__device__ __forceinline__ void dfacc_add_prod(dfacc& a, df x, df y) {
  const float p = __fmul_rn(x.hi, y.hi);
  const float e = __fmaf_rn(x.hi, y.hi, -p);
  const float pl = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
  const df s = two_sum(a.hi, p);
  a.hi = s.hi;
  a.lo = a.lo + (s.lo + pl);
}

// a + b of two accumulators (TwoSum of the high parts, the low parts added)
__device__ __forceinline__ dfacc dfacc_add(dfacc a, dfacc b) {
  const df s = two_sum(a.hi, b.hi);
  dfacc r;
  r.hi = s.hi;
  r.lo = (a.lo + b.lo) + s.lo;
  return r;
}

__device__ __forceinline__ double dfacc_to_double(dfacc a) { return __dadd_rn((double)a.hi, (double)a.lo); }

}  // namespace pg
