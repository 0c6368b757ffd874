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

}  // namespace xt
