// Double-float ("df") arithmetic: an unevaluated sum hi + lo of two FP32
// numbers carrying ~48 significant bits.  On GB300 the FP64 pipe issues at a
// small fraction of the FP32 rate, so the per-particle set-up (square roots,
// quotients, logarithms), the inner products (bilinear interpolation, deposit
// weights, field contractions) of the FP64 path run as df on the FP32 pipe;
// the atomics and final reductions stay in true FP64, fed by exact integer
// float -> double widening.
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

// a + b exactly as a pair (Knuth's TwoSum).
__device__ __forceinline__ df df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v))};
}

// a > b for normalised pairs
__device__ __forceinline__ bool df_gt(df a, df b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }

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

// Lazily renormalised sum of df products (12 FP32 operations a term instead
// of df_fma's 18): s collects the leading product parts through TwoSum, e the
// TwoSum and TwoProd errors and the FP32 cross terms.  (s, e) is not kept
// normalised, |e| stays ~2^-23 |s|, so it may be read directly as a df operand
// of further products (the dropped lo*lo term is ~2^-46 relative); after n
// terms the error is ~n 2^-47 of the sum of |terms|.
struct dacc {
  float s = 0.f, e = 0.f;
  __device__ __forceinline__ void fma(df x, df y) {
    const float p = __fmul_rn(x.h, y.h);
    float pe = __fmaf_rn(x.h, y.h, -p);
    pe = __fmaf_rn(x.h, y.l, pe);
    pe = __fmaf_rn(x.l, y.h, pe);
    const float t = __fadd_rn(s, p);
    const float v = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, v)), __fsub_rn(p, v));
    s = t;
    e = __fadd_rn(e, __fadd_rn(err, pe));
  }
  // fma(x, {yh, yl}) for a table entry whose remainder yl is given unscaled:
  // kl = lo16_unscaled(yh, k), xs = x.h * kLo16Scale (so xs kl = x.h yl)
  __device__ __forceinline__ void fma_lo16(df x, float xs, float yh, float kl) {
    const float p = __fmul_rn(x.h, yh);
    float pe = __fmaf_rn(x.h, yh, -p);
    pe = __fmaf_rn(xs, kl, pe);
    pe = __fmaf_rn(x.l, yh, pe);
    const float t = __fadd_rn(s, p);
    const float v = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, v)), __fsub_rn(p, v));
    s = t;
    e = __fadd_rn(e, __fadd_rn(err, pe));
  }
  // the same state as fma(x, y) from zero (the TwoSum with s = 0 is exact),
  // without the TwoSum
  __device__ __forceinline__ void set(df x, df y) {
    s = __fmul_rn(x.h, y.h);
    float pe = __fmaf_rn(x.h, y.h, -s);
    pe = __fmaf_rn(x.h, y.l, pe);
    e = __fmaf_rn(x.l, y.h, pe);
  }
  __device__ __forceinline__ df raw() const { return {s, e}; }
  __device__ __forceinline__ df value() const { return fast_two_sum(s, e); }
};

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

// Quotient a / b by long division: three FP32 quotient digits, each the
// leading part of the remainder of the previous ones (remainders formed in df)
// times one FP32 reciprocal of b's leading part.  Each digit leaves a
// remainder ~2^-22 of the last, so three digits reach the df rounding level:
// about 2^-46 relative for b away from zero.
__device__ __forceinline__ df df_div(df a, df b) {
  const float rb = __frcp_rn(b.h);
  const float q1 = __fmul_rn(a.h, rb);
  df r = df_sub(a, df_mul({q1, 0.f}, b));
  const float q2 = __fmul_rn(r.h, rb);
  r = df_sub(r, df_mul({q2, 0.f}, b));
  const float q3 = __fmul_rn(r.h, rb);
  return df_add(fast_two_sum(q1, q2), {q3, 0.f});
}

// 1 / sqrt(a) for a > 0: z = the correctly rounded FP32 value, then one
// Newton step z + z (1 - a z^2) / 2 with a z^2 formed in df (z^2 exactly by
// TwoProd); 1 - a z^2 is ~2^-24, so its FP32 value suffices.  About 2^-46
// relative.
__device__ __forceinline__ df df_rsqrt(df a) {
  const float z = __frsqrt_rn(a.h);
  const float p = __fmul_rn(z, z);
  const float e = __fmaf_rn(z, z, -p);            // z*z = p + e exactly
  const df az2 = df_mul(a, {p, e});
  const float d = __fsub_rn(__fsub_rn(1.f, az2.h), az2.l);
  return fast_two_sum(z, __fmul_rn(__fmul_rn(z, d), 0.5f));
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

// ln 2 as a float pair (hi = float rounding of the value, lo = float rounding
// of the remainder).
static __constant__ df kDfLn2 = {0x1.62e430p-1f, -0x1.05c610p-29f};

// Exact float -> double conversion with integer operations, keeping the FP64
// pipe free (every float: zero, normal, infinity and NaN by bit manipulation,
// subnormals through the hardware conversion).
__device__ __forceinline__ double f2d_int(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const unsigned e = (u >> 23) & 0xFF;
  if ((u & 0x7FFFFFFFu) == 0) return __longlong_as_double((long long)sign);   // signed zero
  if (e == 0) return (double)f;                                               // subnormal (rare)
  const unsigned long long bits = sign | ((unsigned long long)(e == 0xFF ? 2047u : e + 896) << 52) |
                                  ((unsigned long long)(u & 0x7FFFFF) << 29);
  return __longlong_as_double((long long)bits);
}

// hi + lo as a double with one FP64 addition and no conversion instructions.
__device__ __forceinline__ double df_to_int(df a) { return f2d_int(a.h) + f2d_int(a.l); }

// Table remainders stored in 16 bits.  A double t is kept as hi = FP32
// rounding of t and k = round((t - hi) / 2^(e-38)), e the exponent of hi:
// |t - hi| <= 2^(e-24), so |k| <= 2^14, and hi + k 2^(e-38) equals t to
// 2^-39 relative.  hi with a biased exponent below 39 (|hi| < 2^-88) keeps
// k = 0, as do |hi| >= 2^113, infinities and NaN.  The scale is built from hi's exponent
// bits and k is converted by the 1.5 * 2^23 magic-number sum (exact for
// |k| < 2^22), so decoding is four integer/FP32 instructions.
constexpr int kLo16Shift = 38;

__device__ __forceinline__ float lo16_decode(float hi, int k) {
  const int b = (__float_as_int(hi) & 0x7f800000) - (kLo16Shift << 23);
  const float kf = __fsub_rn(__int_as_float(0x4B400000 + k), 12582912.f);
  return __fmul_rn(kf, __int_as_float(max(b, 0)));
}

// The remainder without its constant scale, k 2^e (e the exponent of hi):
// lo16_decode(hi, k) = lo16_unscaled(hi, k) 2^-38 exactly.  Exact for
// |hi| < 2^113 (lo16_encode stores no remainder above), 0 for a zero or
// subnormal hi.  A product c lo is then (c 2^-38) (k 2^e), with the 2^-38
// applied to c once per coefficient.
__device__ __forceinline__ float lo16_unscaled(float hi, int k) {
  const float kf = __fsub_rn(__int_as_float(0x4B400000 + k), 12582912.f);
  return __fmul_rn(kf, __int_as_float(__float_as_int(hi) & 0x7f800000));
}
constexpr float kLo16Scale = 0x1.0p-38f;   // 2^-kLo16Shift

__device__ __forceinline__ short lo16_encode(double t, float hi) {
  const int hb = (__float_as_int(hi) >> 23) & 0xff;
  if (hb < kLo16Shift + 1 || hb >= 127 + 113) return 0;   // (also infinities and NaN)
  const double r = t - (double)hi;                       // exact
  return (short)llrint(ldexp(r, 127 + kLo16Shift - hb));  // r / 2^(e-38), exact scaling
}

__device__ __forceinline__ df df_split_or_from(double v) {
  bool ok;
  const df d = df_split(v, ok);
  return ok ? d : df_from(v);
}

}  // namespace xt
