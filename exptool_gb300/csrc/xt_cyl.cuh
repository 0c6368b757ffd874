// Cylindrical EOF basis: device tables and per-point kernels.
//
// Reference: exptool/basis/eof.py (return_bins :354-427, get_pot :430-457,
// accumulate :492-640, force_eval :756-870, accumulated_eval :874-929,
// accumulated_eval_particles :989-1144).
#pragma once

#include <type_traits>

#include "xt_common.cuh"

namespace xt {

template <typename R>
struct CylTab {
  int mmax, norder, numx, numy, cmap;
  R XMIN, dX, YMIN, dY, ascale, hscale;
  R inv_dX, inv_dY, inv_ascale, inv_hscale;
};

// eof.return_bins + bilinear weights (eof.py:354-427, 436-449).  The lower
// clamps zero both index and coordinate; the upper clamps change only the
// index (the coordinate clamp that follows tests the clamped index and never
// fires), so points beyond the last cell are linearly extrapolated.
template <typename R>
struct CylBins {
  int node;       // ix*(numy+1) + iy
  R c00, c10, c01, c11;
};

template <typename R>
__device__ __forceinline__ CylBins<R> cyl_bins(const CylTab<R>& T, R Rcyl, R z) {
  R X = (r_to_xi_inv(Rcyl, T.cmap, T.inv_ascale) - T.XMIN) * T.inv_dX;
  R Y = (z_to_y_inv(z, T.inv_hscale) - T.YMIN) * T.inv_dY;
  R fx = trunc(X), fy = trunc(Y);
  if (!(fx >= R(0))) fx = R(0);       // negative or NaN
  if (!(fy >= R(0))) fy = R(0);
  if (X < R(0)) X = R(0);
  if (Y < R(0)) Y = R(0);
  if (fx >= R(T.numx)) fx = R(T.numx - 1);
  if (fy >= R(T.numy)) fy = R(T.numy - 1);
  const int ix = (int)fx, iy = (int)fy;
  const R delx0 = fx + R(1) - X, dely0 = fy + R(1) - Y;
  const R delx1 = X - fx, dely1 = Y - fy;
  CylBins<R> B;
  B.node = ix * (T.numy + 1) + iy;
  B.c00 = delx0 * dely0;
  B.c10 = delx1 * dely0;
  B.c01 = delx0 * dely1;
  B.c11 = delx1 * dely1;
  return B;
}

struct CylEvalOpts {
  int mode;       // XT_CYL_*
  int m1, m2;     // accumulated_eval_particles m range
  int mmax_use;
  int no_odd;
  int perturb;
  int density;
  int nf;         // fields per (node, m): 6 or 8
};

// Field F: per node, per m, nf values
//   [PC RC ZC PS RS ZS (DC DS)] = sum_n {cos,sin}[m,n] * {pot,rforce,zforce,dens}{C,S}[m,n,node]
// One point with precomputed bins: out = p0 p fr fp fz d0 d fr0 fz0 (mode-specific meaning).
template <typename R>
__device__ __forceinline__ void cyl_eval_bins(const CylTab<R>& T, const R* __restrict__ F, const CylBins<R>& B,
                                              R c1, R s1, const CylEvalOpts& o, R out[9]) {
  const int ny1 = T.numy + 1;
  const int stride = (T.mmax + 1) * o.nf;
  const R* f00 = F + (size_t)B.node * stride;
  const R* f01 = f00 + stride;                 // iy+1
  const R* f10 = f00 + (size_t)ny1 * stride;   // ix+1
  const R* f11 = f10 + stride;
  R p0 = 0, p = 0, fr = 0, fp = 0, fz = 0, d0 = 0, d = 0, fr0 = 0, fz0 = 0;
  R cprev = R(1), sprev = R(0), ccur = c1, scur = s1;   // cos/sin of m phi by recurrence
  const int mtop = o.mmax_use;
#pragma unroll 2
  for (int m = 0; m <= mtop; ++m) {
    R c, s;
    if (m == 0) { c = R(1); s = R(0); }
    else if (m == 1) { c = c1; s = s1; }
    else {
      c = R(2) * c1 * ccur - cprev;
      s = R(2) * c1 * scur - sprev;
      cprev = ccur; sprev = scur; ccur = c; scur = s;
    }
    bool use = true;
    if (o.mode == XT_CYL_ACCUMULATED_EVAL_PARTICLES) use = (m >= o.m1 && m <= o.m2);
    if (o.mode == XT_CYL_ACCUMULATED_EVAL) use = !(o.no_odd && (m & 1));
    if (!use) continue;
    const int b = m * o.nf;
    R v[8];
    // fields in pairs: nf is 6 or 8 and nodes are (mmax+1) nf values apart, so
    // every pair starts at a multiple of two values (one 8- or 16-byte load)
    using R2 = typename std::conditional<std::is_same<R, float>::value, float2, double2>::type;
#pragma unroll
    for (int k = 0; k < 8; k += 2) {
      if (k >= o.nf) break;
      const R2 g00 = *reinterpret_cast<const R2*>(f00 + b + k), g10 = *reinterpret_cast<const R2*>(f10 + b + k);
      const R2 g01 = *reinterpret_cast<const R2*>(f01 + b + k), g11 = *reinterpret_cast<const R2*>(f11 + b + k);
      v[k] = g00.x * B.c00 + g10.x * B.c10 + g01.x * B.c01 + g11.x * B.c11;
      v[k + 1] = g00.y * B.c00 + g10.y * B.c10 + g01.y * B.c01 + g11.y * B.c11;
    }
    const R pm = c * v[0] + s * v[3];
    const R frm = c * v[1] + s * v[4];
    const R fzm = c * v[2] + s * v[5];
    const R fpm = R(m) * (s * v[0] - c * v[3]);
    const R dm = (o.nf == 8) ? (c * v[6] + s * v[7]) : R(0);
    if (o.mode == XT_CYL_FORCE_EVAL) {
      if (m == 0) {
        p0 = pm; fr0 = frm; fz0 = fzm;
      } else {
        // odd-m mask |cos(pi/2 m)| of eof.force_eval (eof.py:822-826)
        const R mask = o.no_odd ? R(fabs(cos((PI / 2.0) * (double)m))) : R(1);
        p += mask * pm; fr += mask * frm; fz += mask * fzm; fp += mask * fpm;
      }
    } else if (o.mode == XT_CYL_ACCUMULATED_EVAL_PARTICLES) {
      if (m == 0) { p0 = pm; d0 = dm; }
      else { p += pm; d += dm; }
      fr += frm; fz += fzm; fp += fpm;
    } else {  // ACCUMULATED_EVAL: totals, with p0/d0 the m = 0 parts
      p += pm; d += dm; fr += frm; fz += fzm; fp += fpm;
      if (m == 0) { p0 = p; d0 = d; }
    }
  }
  out[0] = p0; out[1] = p; out[2] = fr; out[3] = fp; out[4] = fz;
  out[5] = d0; out[6] = d; out[7] = fr0; out[8] = fz0;
}

template <typename R, int MCAP>
__device__ __forceinline__ void cyl_eval_point(const CylTab<R>& T, const R* __restrict__ F, R Rcyl, R z, R c1,
                                               R s1, const CylEvalOpts& o, R out[9]) {
  const CylBins<R> B = cyl_bins(T, Rcyl, z);
  cyl_eval_bins(T, F, B, c1, s1, o, out);
}

}  // namespace xt
