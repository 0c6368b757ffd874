// Double-float ("df") arithmetic: an unevaluated sum hi + lo of two FP32
// numbers carrying ~48 significant bits.  On GB300 the FP64 pipe issues at a
// small fraction of the FP32 rate, so the inner products of the FP64 path
// (bilinear field interpolation, deposit weights) run as df on the FP32 pipe;
// per-particle set-up, atomics and reductions stay in true FP64.
//
// Algorithms: TwoSum (Knuth) and FMA-based TwoProd (exact product error),
// followed by FastTwoSum renormalisation, as in the double-double /
// double-float literature (Dekker 1971; Hida, Li and Bailey, "Library for
// double-double and quad-double arithmetic", 2000).  Relative error per
// operation is ~2^-47 for operands away from the FP32 range limits.
#pragma once

#include <cuda_runtime.h>

namespace xt {

struct __align__(8) df {
  float h, l;
};

__device__ __forceinline__ df df_from(double v) {
  const float h = __double2float_rn(v);
  const float l = __double2float_rn(v - (double)h);
  return {h, l};
}

__device__ __forceinline__ double df_to(df a) { return (double)a.h + (double)a.l; }

__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

__device__ __forceinline__ df df_add(df a, df b) {
  const float s = __fadd_rn(a.h, b.h);
  const float v = __fsub_rn(s, a.h);
  const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, v)), __fsub_rn(b.h, v));
  const float t = __fadd_rn(e, __fadd_rn(a.l, b.l));
  return fast_two_sum(s, t);
}

__device__ __forceinline__ df df_neg(df a) { return {-a.h, -a.l}; }

__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return fast_two_sum(p, e);
}

// a * b + c with one renormalisation.
__device__ __forceinline__ df df_fma(df a, df b, df c) { return df_add(df_mul(a, b), c); }

// multiply by a small exact float (an integer m or 2)
__device__ __forceinline__ df df_scale(df a, float s) {
  const float p = __fmul_rn(a.h, s);
  float e = __fmaf_rn(a.h, s, -p);
  e = __fmaf_rn(a.l, s, e);
  return fast_two_sum(p, e);
}

// Square root of a >= 0: y = sqrt(a.h) in FP32, then one correction
// y + (a - y^2) / (2y) with y^2 formed exactly (Karp & Markstein's
// refinement); about 2^-46 relative.
__device__ __forceinline__ df df_sqrt(df a) {
  if (!(a.h > 0.f)) return {0.f, 0.f};
  const float y = __fsqrt_rn(a.h);
  const float p = __fmul_rn(y, y);
  const float e = __fmaf_rn(y, y, -p);          // y*y = p + e exactly
  const df r = df_sub(a, {p, e});
  return fast_two_sum(y, __fdiv_rn(r.h, __fmul_rn(2.f, y)));
}

// Quotient a / b by long division: three FP32 quotient digits, each from the
// remainder of the previous ones (remainders formed in df); about 2^-46
// relative for b away from zero.
__device__ __forceinline__ df df_div(df a, df b) {
  const float q1 = __fdiv_rn(a.h, b.h);
  df r = df_sub(a, df_mul({q1, 0.f}, b));
  const float q2 = __fdiv_rn(r.h, b.h);
  r = df_sub(r, df_mul({q2, 0.f}, b));
  const float q3 = __fdiv_rn(r.h, b.h);
  return df_add(fast_two_sum(q1, q2), {q3, 0.f});
}

__device__ __forceinline__ df df_abs(df a) { return a.h < 0.f ? df_neg(a) : a; }

// Split of a double into a float pair with integer operations only (no
// FP64 conversion instructions): hi = the leading 24 significand bits
// (truncated), lo = the next 24 of the remaining 29 (truncated), so
// hi + lo = v to 2^-47 relative and |lo| < ulp(hi).  Valid for
// 2^-74 <= |v| < 2^127; zero returns (0, 0); ok = false outside that range
// (callers then use df_from).
__device__ __forceinline__ df df_split(double v, bool& ok) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned sign = (unsigned)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7FF);
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  ok = true;
  if (e == 0 && m == 0) return {__uint_as_float(sign), 0.f};
  if (e < 949 || e > 1149) {
    ok = false;
    return {0.f, 0.f};
  }
  const float hi = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | (unsigned)(m >> 29));
  const unsigned rem = (unsigned)(m & 0x1FFFFFFFull);      // value rem * 2^(e - 1075)
  if (rem == 0) return {hi, 0.f};
  const int pos = 31 - __clz((int)rem);                     // leading one, 0..28
  const unsigned mant = pos > 23 ? (rem >> (pos - 23)) : (rem << (23 - pos));
  const float lo = __uint_as_float(sign | ((unsigned)(pos + e - 948) << 23) | (mant & 0x7FFFFFu));
  return {hi, lo};
}

__device__ __forceinline__ df df_split_or_from(double v) {
  bool ok;
  const df d = df_split(v, ok);
  return ok ? d : df_from(v);
}

}  // namespace xt
