// FP64 spherical (SL) evaluation in double-float arithmetic.
//
// spheresl.all_eval / all_eval_particles / force_eval (spheresl.py:987,
// 1107-1234, 1240-1362) at FP64 accuracy without the FP64 pipe, which on
// GB300 issues at a small fraction of the FP32 rate: cos theta and
// cos/sin phi, the lerp and force-stencil weights of sph_bins
// (spheresl.py:106-160), the Legendre values and derivatives
// (spheresl.py:664-770), the azimuthal multiples (spheresl.py:773-796) and
// every sum of the field contraction run as double-float ("df", hi + lo FP32
// pairs) on the FP32 pipe.  The radius, the radial map with its clamps, the
// node and the in-cell offsets stay FP64 (a few operations per point; see
// sph_bins_df).  The FP64 field
// values and table entries are split into float pairs with integer
// operations; only the seven outputs are widened to FP64.  The order of the
// operations is the one of sph_eval_point<double> (xt_sph.cuh), each rounded
// to ~2^-47 instead of 2^-53.
//
// Points whose coordinates leave the range where FP32 exponents are safe
// (|x|, |y|, |z| >= 1e15, or below 2^-74 without being 0, or NaN), points on
// the z axis (rho^2 < 1e-30, where cos/sin phi come from atan2) and
// spherical-coordinate input (phi given, so sincos is needed) take the FP64
// arithmetic of sph_eval_point<double> instead.
#include <cmath>

#include "xt_df.cuh"
#include "xt_internal.cuh"
#include "xt_launch.cuh"

namespace xt {

// 1 / k for k = 0..16 as float pairs (k = 0 unused).
struct SphDfInv {
  df v[17];
};

// Table constants as float pairs, split on the host.
struct SphDfConst {
  df inv_scale, xi0, inv_dxi, lo, hi;
  df half_inv_scale;            // 0.5 / scale (cmap 1 force factor)
  df exp_neg_lo, exp_neg_hi;    // exp(-lo), exp(-hi) (cmap 2 force factor at the clamps)
  df one_m_eps;                 // 1 - 1e-8 (cmap 1 clamp, dlegendre pole clamp)
  SphDfInv inv;
};

__device__ __forceinline__ bool df_lt(df a, df b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
__device__ __forceinline__ bool df_finite(df a) { return isfinite(a.h) && isfinite(a.l); }
__device__ __forceinline__ df dfs(double v) { return df_split_or_from(v); }

// sph_bins (spheresl.py:121-160) for one radius.
struct SphBinsDf {
  int i, j;
  df wp[3], wd[3];
  df fac, x2;     // force = fac (D1[j] + x2 D2[j]) from the field's differences
};

// The map, its clamps, the node and the in-cell offsets x1, x2 are FP64,
// exactly as sph_bins<double>: x2 multiplies the node spacing's inverse
// (~1e2 to 1e3) and the table's steepness, so an absolute error of 1e-13 in
// x = log r (what a double-float logarithm leaves) became 1e-11 relative in
// the densities and 2e-10 in the radial force.  About 35 FP64 operations per
// point, on the FP64 pipe alongside the FP32 work; everything after x1, x2 is
// double-float.
__device__ __forceinline__ SphBinsDf sph_bins_df(const SphTab<double>& T, const SphDfConst& K, double r64, df r,
                                                 bool need_dens) {
  const df one{1.f, 0.f};
  double x = r_to_xi_inv(r64, T.cmap, T.inv_scale);
  bool clamp_lo = false, clamp_hi = false;
  if (T.cmap == 1) {
    if (x < -1.0) x = -1.0;
    if (x >= 1.0) x = 1.0 - 1.0e-08;
  }
  if (T.cmap == 2) {
    if (x < T.lo) {
      x = T.lo;
      clamp_lo = true;
    }
    if (x > T.hi) {
      x = T.hi;
      clamp_hi = true;
    }
  }
  double fi = floor((x - T.xi0) * T.inv_dxi);
  if (!(fi >= 0.0)) fi = 0.0;
  if (fi > (double)(T.numr - 2)) fi = (double)(T.numr - 2);
  const int i = (int)fi;
  const df x1 = dfs((T.xi[i + 1] - x) * T.inv_dxi);
  const df x2 = dfs((x - T.xi[i]) * T.inv_dxi);
  const df xd = dfs(x);
  SphBinsDf B;
  const int j = i < 1 ? 1 : i;
  B.i = i;
  B.j = j;
  const df plerp = df_add(df_mul(x1, dfs(T.p0[i])), df_mul(x2, dfs(T.p0[i + 1])));
  const df lw0 = df_mul(x1, plerp), lw1 = df_mul(x2, plerp);
  const df zero{0.f, 0.f};
  if (i == j) {
    B.wp[0] = zero; B.wp[1] = lw0; B.wp[2] = lw1;
  } else {
    B.wp[0] = lw0; B.wp[1] = lw1; B.wp[2] = zero;
  }
  // d xi / dr / dxi (compatibility.d_xi_to_r, compatibility.py:65-80)
  df fac;
  if (T.cmap == 1) {
    const df d = df_sub(one, xd);
    fac = df_mul(df_mul(df_mul(d, d), K.half_inv_scale), K.inv_dxi);
  } else if (T.cmap == 2) {
    // exp(-x) = 1 / r where x = log r is not clamped
    const df e = clamp_lo ? K.exp_neg_lo : (clamp_hi ? K.exp_neg_hi : df_div(one, r));
    fac = df_mul(e, K.inv_dxi);
  } else {
    fac = K.inv_dxi;
  }
  B.fac = fac;
  B.x2 = x2;
  if (need_dens) {
    const df dlerp = df_add(df_mul(x1, dfs(T.d0[i])), df_mul(x2, dfs(T.d0[i + 1])));
    const df a0 = df_mul(x1, dlerp), a1 = df_mul(x2, dlerp);
    if (i == j) {
      B.wd[0] = zero; B.wd[1] = a0; B.wd[2] = a1;
    } else {
      B.wd[0] = a0; B.wd[1] = a1; B.wd[2] = zero;
    }
  } else {
    B.wd[0] = B.wd[1] = B.wd[2] = zero;
  }
  return B;
}

// One point: out = den0 den1 pot0 pot1 potr pott potp, as sph_eval_point.
// The Legendre values are generated degree by degree with the recurrences of
// legendre() (sectoral P_l^l = -(2l-1) somx2 P_{l-1}^{l-1}, P_l^{l-1} =
// (2l-1) x P_{l-1}^{l-1}, and the three-term recurrence in l), keeping only
// degrees l-1 and l-2, and each dP_l^m of dlegendre() is formed where it is
// used: the same values as the full triangles, in a third of the registers.
template <int LCAP>
__device__ __forceinline__ void sph_eval_point_df(const SphTab<double>& T, const SphDfConst& K,
                                                  const double* __restrict__ GH, double r64, df r, df costh, df c1,
                                                  df s1, const SphEvalOpts& o, double out[7]) {
  const int lmax = o.lmax_use;
  const int nrow = sph_nrow(T.lmax);
  const bool dens = o.want_dens;
  const df one{1.f, 0.f}, zero{0.f, 0.f};
  const SphBinsDf B = sph_bins_df(T, K, r64, r, dens);
  const df x = costh;
  const df somx2 = df_sqrt(df_mul(df_sub(one, x), df_add(one, x)));   // 0 where |x| > 1 by rounding
  // dlegendre: x clamped to +-(1 - 1e-8) (1 - |x| < 1e-8), sd = 1 / (x^2 - 1)
  const df xc = df_lt(K.one_m_eps, df_abs(x)) ? (x.h > 0.f ? K.one_m_eps : df_neg(K.one_m_eps)) : x;
  const df sd = df_div(one, df_sub(df_mul(xc, xc), one));
  auto fin = [](df v) { return df_finite(v) ? v : df{0.f, 0.f}; };
  df cm[LCAP + 1], sm[LCAP + 1];
  cm[0] = one;
  sm[0] = zero;
  if (LCAP >= 1) {
    cm[1] = c1;
    sm[1] = s1;
  }
  const df c2 = df_scale(c1, 2.f);
#pragma unroll
  for (int k = 2; k <= LCAP; ++k) {
    if (k > lmax) break;
    cm[k] = df_sub(df_mul(c2, cm[k - 1]), cm[k - 2]);
    sm[k] = df_sub(df_mul(c2, sm[k - 1]), sm[k - 2]);
  }
  constexpr int PR = SphFieldLayout<double>::per_row;   // G, Gd, D1, D2
  const double* g0 = GH + (size_t)(B.j - 1) * nrow * PR;
  const double* g1 = g0 + nrow * PR;
  const double* g2 = g1 + nrow * PR;
  auto rowvals = [&](int row, df& pot, df& frc, df& den) {
    const df a0 = dfs(g0[PR * row]), a1 = dfs(g1[PR * row]), a2 = dfs(g2[PR * row]);
    dacc p, f;
    p.set(B.wp[0], a0);
    p.fma(B.wp[1], a1);
    p.fma(B.wp[2], a2);
    // fac ((H[j+1]-H[j-1])/2 + x2 (H[j-1]-2H[j]+H[j+1])), the differences
    // taken in FP64 by the field kernel
    f.set(B.x2, dfs(g1[PR * row + 3]));
    f.fma(one, dfs(g1[PR * row + 2]));
    pot = p.raw();
    frc = df_mul(B.fac, f.raw());
    if (dens) {
      const df b0 = dfs(g0[PR * row + 1]), b1 = dfs(g1[PR * row + 1]), b2 = dfs(g2[PR * row + 1]);
      dacc d;
      d.set(B.wd[0], b0);
      d.fma(B.wd[1], b1);
      d.fma(B.wd[2], b2);
      den = d.raw();
    } else {
      den = zero;
    }
  };
  const df f00 = dfs(T.fact[0]);
  df pot, frc, den;
  rowvals(0, pot, frc, den);
  const df den0 = df_mul(f00, den), pot0 = df_mul(f00, pot);
  dacc den1, pot1, potr, pott, potp;
  potr.set(f00, frc);
  if (o.mode == XT_SPH_ALL_EVAL) {
    den1.s = den0.h;
    den1.e = den0.l;
  }
  const int lstride = T.lmax + 1;
  df P1[LCAP + 1], P2[LCAP + 1];               // P_{l-1}^m, P_{l-2}^m
#pragma unroll
  for (int m = 0; m <= LCAP; ++m) P1[m] = P2[m] = zero;
  P1[0] = one;                                 // P_0^0
  df P10{0.f, 0.f};                            // P_1^0, the den1 factor of all_eval_particles
#pragma unroll
  for (int l = 1; l <= LCAP; ++l) {
    if (l > lmax) break;
    df Pl[LCAP + 1];
#pragma unroll
    for (int m = 0; m <= LCAP; ++m) Pl[m] = zero;
    const df xl = df_scale(x, (float)(2 * l - 1));
#pragma unroll
    for (int m = 0; m <= l; ++m) {
      if (m == l) Pl[m] = df_mul(df_scale(P1[l - 1], -(float)(2 * l - 1)), somx2);
      else if (m == l - 1) Pl[m] = df_mul(xl, P1[m]);
      else Pl[m] = df_mul(df_sub(df_mul(xl, P1[m]), df_scale(P2[m], (float)(l + m - 1))), K.inv.v[l - m]);
    }
    if (l == 1) P10 = fin(Pl[0]);
    const bool skip = (o.mode == XT_SPH_ALL_EVAL_PARTICLES && (l > o.L2 || l < o.L1)) || (o.no_odd && (l & 1));
    if (!skip) {
      const int loff = l * l;
      const df xcl = df_scale(xc, (float)l);
      {  // m = 0
        const df f = dfs(T.fact[l * lstride]);
        rowvals(loff, pot, frc, den);
        const df P = fin(Pl[0]);
        const df dP = fin(df_mul(sd, df_sub(df_mul(xcl, P), df_scale(fin(P1[0]), (float)l))));
        const df fP = df_mul(f, P);
        if (dens) den1.fma(df_mul(f, (o.mode == XT_SPH_ALL_EVAL_PARTICLES) ? P10 : P), den);
        pot1.fma(fP, pot);
        potr.fma(fP, frc);
        pott.fma(df_mul(f, dP), pot);
      }
#pragma unroll
      for (int m = 1; m <= l; ++m) {
        const df f = dfs(T.fact[l * lstride + m]);
        df potc, frcc, denc, pots, frcs, dens_;
        rowvals(loff + 2 * m - 1, potc, frcc, denc);
        rowvals(loff + 2 * m, pots, frcs, dens_);
        const int k = o.trig_l ? l : m;
        const df c = cm[k], s = sm[k];
        const df P = fin(Pl[m]);
        const df dP = m < l ? fin(df_mul(sd, df_sub(df_mul(xcl, P), df_scale(fin(P1[m]), (float)(l + m)))))
                            : fin(df_mul(df_mul(sd, xcl), P));
        const df fP = df_mul(f, P);
        dacc ap;
        ap.set(potc, c);
        ap.fma(pots, s);
        const df angp = ap.raw();
        if (dens) {
          dacc ad;
          ad.set(denc, c);
          ad.fma(dens_, s);
          den1.fma(fP, ad.raw());
        }
        pot1.fma(fP, angp);
        dacc af;
        af.set(frcc, c);
        af.fma(frcs, s);
        potr.fma(fP, af.raw());
        pott.fma(df_mul(f, dP), angp);
        dacc aq;
        aq.set(df_neg(potc), s);
        aq.fma(pots, c);
        potp.fma(df_scale(fP, (float)m), aq.raw());
      }
    }
#pragma unroll
    for (int m = 0; m <= LCAP; ++m) {
      P2[m] = P1[m];
      P1[m] = Pl[m];
    }
  }
  out[0] = df_to(den0);
  out[1] = df_to(den1.value());
  out[2] = df_to(pot0);
  out[3] = df_to(pot1.value());
  out[4] = df_to(potr.value());
  out[5] = df_to(pott.value());
  out[6] = df_to(potp.value());
}

template <int LCAP>
__global__ void __launch_bounds__(128) k_sph_eval_df(SphTab<double> T, SphDfConst K, const double* __restrict__ GH,
                                                     int coord_mode, const double* __restrict__ a,
                                                     const double* __restrict__ b, const double* __restrict__ c,
                                                     long long n, SphEvalOpts o, double* o0, double* o1, double* o2,
                                                     double* o3, double* o4, double* o5, double* o6, double* o7) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    double v[7];
    double rr = 0.0;
    bool done = false;
    if (coord_mode == XT_COORD_CART) {
      const double xx = a[p], yy = b[p], zz = c[p];
      bool okx, oky, okz;
      const df xd = df_split(xx, okx), yd = df_split(yy, oky), zd = df_split(zz, okz);
      const df s2 = df_add(df_mul(xd, xd), df_mul(yd, yd));
      const bool safe = okx && oky && okz && fabsf(xd.h) < 1.0e15f && fabsf(yd.h) < 1.0e15f &&
                        fabsf(zd.h) < 1.0e15f && s2.h > 1.0e-30f;
      if (safe) {
        const double r64 = sqrt(xx * xx + yy * yy + zz * zz);
        const df r = dfs(r64);
        const df irho = df_rsqrt(s2);             // cos, sin phi = x, y / rho
        const df costh = df_div(zd, r);
        sph_eval_point_df<LCAP>(T, K, GH, r64, r, costh, df_mul(xd, irho), df_mul(yd, irho), o, v);
        if (o7) rr = df_to(df_sqrt(s2));
        done = true;
      }
    }
    if (!done) {
      // FP64 arithmetic: spherical-coordinate input and the points above
      double r, costh, c1, s1;
      if (coord_mode == XT_COORD_CART) {
        const double xx = a[p], yy = b[p], zz = c[p];
        r = sqrt(xx * xx + yy * yy + zz * zz);
        rr = sqrt(xx * xx + yy * yy);
        costh = zz / r;
        unit_phi(xx, yy, c1, s1);
      } else {
        r = a[p];
        costh = b[p];
        sincos_r(c[p], &s1, &c1);
      }
      sph_eval_point<double, LCAP>(T, GH, r, costh, c1, s1, o, v);
    }
    if (o.mode == XT_SPH_FORCE_EVAL) {
      // potr pott potp pot1 pot0
      if (o0) o0[p] = v[4];
      if (o1) o1[p] = v[5];
      if (o2) o2[p] = v[6];
      if (o3) o3[p] = v[3];
      if (o4) o4[p] = v[2];
    } else {
      const double densfac = (o.mode == XT_SPH_ALL_EVAL_PARTICLES) ? 0.25 * PI : 0.25 / PI;
      if (o0) o0[p] = v[0] * densfac;
      if (o1) o1[p] = v[1] * densfac;
      if (o2) o2[p] = v[2];
      if (o3) o3[p] = v[3];
      if (o4) o4[p] = v[4];
      if (o5) o5[p] = v[5];
      if (o6) o6[p] = v[6];
      if (o7 && o.mode == XT_SPH_ALL_EVAL_PARTICLES) o7[p] = rr;
    }
  }
}

static df host_df_pair(double v) {
  const float h = (float)v;
  return {h, (float)(v - (double)h)};
}

static SphDfConst sph_df_const(const SphTab<double>& T) {
  SphDfConst K;
  K.inv_scale = host_df_pair(T.inv_scale);
  K.xi0 = host_df_pair(T.xi0);
  K.inv_dxi = host_df_pair(T.inv_dxi);
  K.lo = host_df_pair(T.lo);
  K.hi = host_df_pair(T.hi);
  K.half_inv_scale = host_df_pair(0.5 / T.scale);
  K.exp_neg_lo = host_df_pair(std::exp(-T.lo));
  K.exp_neg_hi = host_df_pair(std::exp(-T.hi));
  K.one_m_eps = host_df_pair(1.0 - 1.0e-8);
  K.inv.v[0] = {0.f, 0.f};
  for (int k = 1; k <= 16; ++k) K.inv.v[k] = host_df_pair(1.0 / (double)k);
  return K;
}

template <int LC>
void launch_sph_eval_df(const SphTab<double>& T, const double* GH, int coord_mode, const double* a, const double* b,
                        const double* c, long long n, const SphEvalOpts& o, double* const* outs, cudaStream_t st) {
  const SphDfConst K = sph_df_const(T);
  const int grid = resident_grid(k_sph_eval_df<LC>, 128, 0, n);
  k_sph_eval_df<LC><<<grid, 128, 0, st>>>(T, K, GH, coord_mode, a, b, c, n, o, outs[0], outs[1], outs[2], outs[3],
                                         outs[4], outs[5], outs[6], outs[7]);
}

template void launch_sph_eval_df<4>(const SphTab<double>&, const double*, int, const double*, const double*,
                                    const double*, long long, const SphEvalOpts&, double* const*, cudaStream_t);
template void launch_sph_eval_df<6>(const SphTab<double>&, const double*, int, const double*, const double*,
                                    const double*, long long, const SphEvalOpts&, double* const*, cudaStream_t);
template void launch_sph_eval_df<8>(const SphTab<double>&, const double*, int, const double*, const double*,
                                    const double*, long long, const SphEvalOpts&, double* const*, cudaStream_t);

}  // namespace xt
