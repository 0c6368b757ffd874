// Spherical Sturm-Liouville basis: device tables and per-point kernels.
//
// Reference: exptool/basis/spheresl.py (accumulation :567-656, evaluation
// :987-1362, radial functions :106-335, Legendre :664-770).
#pragma once

#include <type_traits>

#include "xt_common.cuh"

namespace xt {

// Device view of an uploaded SL table.  Arrays in precision R (double for
// the drop-in path, float for the mixed path).
template <typename R>
struct SphTab {
  int lmax, nmax, numr, cmap;
  R scale, xi0, dxi, lo, hi;   // xi0 = min(xi), dxi = xi[1]-xi[0]; lo/hi: cmap=2 clamp
  R inv_scale, inv_dxi;
  const R* xi;                 // [numr]
  const R* p0;                 // [numr]  model potential on the grid
  const R* d0;                 // [numr]  4 pi rho0 on the grid
  const R* fact;               // [(lmax+1)^2] factorial_return, index l*(lmax+1)+m
  const R* rnode;              // [numr] node radii xi_to_r(xi) (FP32 path: accurate in-cell offsets)
};

__host__ __device__ inline int sph_nrow(int lmax) { return (lmax + 1) * (lmax + 1); }
__host__ __device__ inline int tri(int l, int m) { return l * (l + 1) / 2 + m; }

// Radial interpolation set-up of get_halo_* (spheresl.py:121-143): mapped
// coordinate, clamp, node index and linear weights.  Returns the 3-node
// stencil base j = max(indx, 1) and weights such that, for any per-node
// quantity G,
//   pot-like   lerp(G) * plerp  = wp[0] G[j-1] + wp[1] G[j] + wp[2] G[j+1]
//   force-like fac*(stencil)    = wf[0] G[j-1] + wf[1] G[j] + wf[2] G[j+1]
//   dens-like  lerp(G) * dlerp  = wd[0] G[j-1] + wd[1] G[j] + wd[2] G[j+1]
// The force stencil at indx == 0 uses rows 0,1,2 with the unshifted x2
// (spheresl.py:147-150).  With H = p0 G the stencil is
//   fac * ( (H[j+1]-H[j-1])/2 + x2 (H[j-1] - 2 H[j] + H[j+1]) ),
// which the FP32 field stores pre-differenced (in FP64), so the FP32 path
// never subtracts nearly equal table values.
template <typename R>
struct SphBins {
  int i, j;       // lerp base node i, stencil centre j = max(i, 1)
  R lw0, lw1;     // x1*plerp, x2*plerp on nodes i, i+1
  R dw0, dw1;     // x1*dlerp, x2*dlerp on nodes i, i+1
  R wp[3], wf[3], wd[3];
  R fac, x2;      // d xi/dr / dxi and the in-cell offset (pre-differenced force)
};

// Coefficient-contracted SL fields.  FP64 (the drop-in path): per node, per
// row, (G, Gd) = sum_n c[row,n] ef[l,n,node] {1/sqrt(ev), sqrt(ev)}.
// FP32 (the mixed path), laid out for one 16-byte gather per row: a float4
// array [numr][nrow] of (G[i], G[i+1], D1[j], D2[j]) with j = max(i, 1),
// D1 = (H[j+1]-H[j-1])/2, D2 = H[j-1]-2H[j]+H[j+1], H = p0 G (all from FP64
// sums), followed by a float2 array [numr][nrow] of (Gd[i], Gd[i+1]).
template <typename R>
struct SphFieldLayout {
  static constexpr bool f32 = std::is_same<R, float>::value;
  // elements of R per (node, row)
  static constexpr int per_row = f32 ? 6 : 2;
};

template <typename R>
__device__ __forceinline__ SphBins<R> sph_bins(const SphTab<R>& T, R r, bool need_force, bool need_dens) {
  R x = r_to_xi_inv(r, T.cmap, T.inv_scale);
  if (T.cmap == 1) {
    if (x < R(-1)) x = R(-1);
    if (x >= R(1)) x = R(1) - R(1.0e-08);
  }
  if (T.cmap == 2) {
    if (x < T.lo) x = T.lo;
    if (x > T.hi) x = T.hi;
  }
  R fi = floor((x - T.xi0) * T.inv_dxi);
  if (!(fi >= R(0))) fi = R(0);                 // negative or NaN
  if (fi > R(T.numr - 2)) fi = R(T.numr - 2);
  int i = (int)fi;
  R x1 = (T.xi[i + 1] - x) * T.inv_dxi;
  R x2 = (x - T.xi[i]) * T.inv_dxi;
  if constexpr (std::is_same<R, float>::value) {
    // FP32: x carries an absolute rounding of ~ulp(x), a sizeable fraction of
    // a table cell; take the in-cell offset from the radius ratio instead,
    // which FP32 resolves to its relative precision.
    const bool clamped = (T.cmap == 2) ? (x == T.lo || x == T.hi) : (T.cmap == 1 && (x == R(-1) || x >= R(1) - R(2.0e-8)));
    if (!clamped && r > R(0)) {
      const R ri = T.rnode[i];
      R dx;
      if (T.cmap == 2) dx = log(r / ri);
      else if (T.cmap == 1) dx = R(2) * (r - ri) * T.inv_scale / ((r * T.inv_scale + R(1)) * (ri * T.inv_scale + R(1)));
      else dx = r - ri;
      x2 = dx * T.inv_dxi;
      x1 = R(1) - x2;
    }
  }
  SphBins<R> B;
  int j = i < 1 ? 1 : i;
  B.i = i;
  B.j = j;
  R plerp = x1 * T.p0[i] + x2 * T.p0[i + 1];
  B.lw0 = x1 * plerp;
  B.lw1 = x2 * plerp;
  if (i == j) {
    B.wp[0] = R(0); B.wp[1] = B.lw0; B.wp[2] = B.lw1;
  } else {
    B.wp[0] = B.lw0; B.wp[1] = B.lw1; B.wp[2] = R(0);
  }
  B.fac = R(0);
  B.x2 = x2;
  B.wf[0] = B.wf[1] = B.wf[2] = R(0);
  if (need_force) {
    const R fac = d_xi_to_r(x, T.cmap, T.scale) * T.inv_dxi;
    B.fac = fac;
    if constexpr (!std::is_same<R, float>::value) {
      B.wf[0] = fac * (x2 - R(0.5)) * T.p0[j - 1];
      B.wf[1] = fac * (R(-2) * x2) * T.p0[j];
      B.wf[2] = fac * (x2 + R(0.5)) * T.p0[j + 1];
    }
  }
  B.dw0 = B.dw1 = R(0);
  if (need_dens) {
    R dlerp = x1 * T.d0[i] + x2 * T.d0[i + 1];
    B.dw0 = x1 * dlerp;
    B.dw1 = x2 * dlerp;
    if (i == j) {
      B.wd[0] = R(0); B.wd[1] = x1 * dlerp; B.wd[2] = x2 * dlerp;
    } else {
      B.wd[0] = x1 * dlerp; B.wd[1] = x2 * dlerp; B.wd[2] = R(0);
    }
  } else {
    B.wd[0] = B.wd[1] = B.wd[2] = R(0);
  }
  return B;
}

// Associated Legendre P_l^m(x) (Condon-Shortley phase) by the recurrences of
// spheresl.legendre_R (spheresl.py:664-700); non-finite values set to 0.
// Stored triangularly: P[tri(l,m)].
template <typename R, int LCAP>
__device__ __forceinline__ void legendre(R x, int lmax, R* P) {
  P[0] = R(1);
  R pll = R(1);
  if (lmax > 0) {
    R somx2 = sqrt((R(1) - x) * (R(1) + x));
    R fact = R(1);
#pragma unroll
    for (int m = 1; m <= LCAP; ++m) {
      if (m > lmax) break;
      pll *= -fact * somx2;
      P[tri(m, m)] = pll;
      fact += R(2);
    }
  }
#pragma unroll
  for (int m = 0; m < LCAP; ++m) {
    if (m >= lmax) break;
    R pl2 = P[tri(m, m)];
    R pl1 = x * R(2 * m + 1) * pl2;
    P[tri(m + 1, m)] = pl1;
#pragma unroll
    for (int l = m + 2; l <= LCAP; ++l) {
      if (l > lmax) break;
      R v = (x * R(2 * l - 1) * pl1 - R(l + m - 1) * pl2) * (R(1) / R(l - m));
      P[tri(l, m)] = v;
      pl2 = pl1;
      pl1 = v;
    }
  }
#pragma unroll
  for (int k = 0; k < (LCAP + 1) * (LCAP + 2) / 2; ++k)
    if (!finite(P[k])) P[k] = R(0);
}

// dP_l^m/dx of spheresl.dlegendre_R (spheresl.py:745-768): x clamped to
// +-(1-1e-8) for the derivative only.
template <typename R, int LCAP>
__device__ __forceinline__ void dlegendre(R x, int lmax, const R* P, R* dP) {
  const R MINEPS = R(1.0e-8);
  if (R(1) - fabs(x) < MINEPS) x = (x > R(0)) ? (R(1) - MINEPS) : -(R(1) - MINEPS);
  R somx2 = R(1) / (x * x - R(1));
  dP[0] = R(0);
#pragma unroll
  for (int l = 1; l <= LCAP; ++l) {
    if (l > lmax) break;
#pragma unroll
    for (int m = 0; m < l; ++m) dP[tri(l, m)] = somx2 * (x * R(l) * P[tri(l, m)] - R(l + m) * P[tri(l - 1, m)]);
    dP[tri(l, l)] = somx2 * x * R(l) * P[tri(l, l)];
  }
#pragma unroll
  for (int k = 0; k < (LCAP + 1) * (LCAP + 2) / 2; ++k)
    if (!finite(dP[k])) dP[k] = R(0);
}

// cos(k phi), sin(k phi), k = 0..kmax, from cos/sin of phi by the Chebyshev
// recurrence of spheresl.sinecosine_R (spheresl.py:773-796).
template <typename R, int LCAP>
__device__ __forceinline__ void multiples(R c1, R s1, int kmax, R* c, R* s) {
  c[0] = R(1);
  s[0] = R(0);
  if (LCAP >= 1) {
    c[1] = c1;
    s[1] = s1;
  }
#pragma unroll
  for (int k = 2; k <= LCAP; ++k) {
    if (k > kmax) break;
    c[k] = R(2) * c1 * c[k - 1] - c[k - 2];
    s[k] = R(2) * c1 * s[k - 1] - s[k - 2];
  }
}

struct SphEvalOpts {
  int mode;      // XT_SPH_*
  int L1, L2;    // all_eval_particles l range
  int no_odd;
  int lmax_use;
  int trig_l;    // azimuthal factor of row (l,m): 1 = cos(l phi) (force_eval), 0 = cos(m phi)
  int want_dens;
};

// One point of the spherical evaluation.  Field GH: per node, per row, the
// coefficient-contracted radial functions in the SphFieldLayout of R.
// out: den0 den1 pot0 pot1 potr pott potp (before the mode's output mapping).
template <typename R, int LCAP>
__device__ __forceinline__ void sph_eval_point(const SphTab<R>& T, const R* __restrict__ GH, R r, R costh, R c1,
                                               R s1, const SphEvalOpts& o, R out[7]) {
  const int lmax = o.lmax_use;
  const int nrow = sph_nrow(T.lmax);
  const bool dens = o.want_dens;
  SphBins<R> B = sph_bins(T, r, true, dens);
  constexpr int NT = (LCAP + 1) * (LCAP + 2) / 2;
  R P[NT], dP[NT];
#pragma unroll
  for (int k = 0; k < NT; ++k) { P[k] = R(0); dP[k] = R(0); }
  legendre<R, LCAP>(costh, lmax, P);
  dlegendre<R, LCAP>(costh, lmax, P, dP);
  R cm[LCAP + 1], sm[LCAP + 1];
  multiples<R, LCAP>(c1, s1, lmax, cm, sm);
  const R* g0 = GH + (size_t)(B.j - 1) * nrow * 2;
  const R* g1 = g0 + nrow * 2;
  const R* g2 = g1 + nrow * 2;

  auto rowvals = [&](int row, R& pot, R& frc, R& den) {
    if constexpr (SphFieldLayout<R>::f32) {
      const float4 q = reinterpret_cast<const float4*>(GH)[(size_t)B.i * nrow + row];
      pot = B.lw0 * q.x + B.lw1 * q.y;
      frc = B.fac * fmaf(B.x2, q.w, q.z);
      if (dens) {
        const float2 d = reinterpret_cast<const float2*>(GH + (size_t)T.numr * nrow * 4)[(size_t)B.i * nrow + row];
        den = B.dw0 * d.x + B.dw1 * d.y;
      } else {
        den = R(0);
      }
    } else {
      R a0 = g0[2 * row], a1 = g1[2 * row], a2 = g2[2 * row];
      pot = B.wp[0] * a0 + B.wp[1] * a1 + B.wp[2] * a2;
      frc = B.wf[0] * a0 + B.wf[1] * a1 + B.wf[2] * a2;
      if (dens) {
        R b0 = g0[2 * row + 1], b1 = g1[2 * row + 1], b2 = g2[2 * row + 1];
        den = B.wd[0] * b0 + B.wd[1] * b1 + B.wd[2] * b2;
      } else {
        den = R(0);
      }
    }
  };

  const R f00 = T.fact[0];
  R pot, frc, den;
  rowvals(0, pot, frc, den);
  R den0 = f00 * den, pot0 = f00 * pot, potr = f00 * frc;
  R den1 = (o.mode == XT_SPH_ALL_EVAL) ? den0 : R(0);
  R pot1 = R(0), pott = R(0), potp = R(0);
  const int lstride = T.lmax + 1;
#pragma unroll
  for (int l = 1; l <= LCAP; ++l) {
    if (l > lmax) break;
    if (o.mode == XT_SPH_ALL_EVAL_PARTICLES && (l > o.L2 || l < o.L1)) continue;
    if (o.no_odd && (l & 1)) continue;
    const int loff = l * l;
    {  // m = 0
      const R f = T.fact[l * lstride];
      rowvals(loff, pot, frc, den);
      const R fP = f * P[tri(l, 0)];
      if (dens) den1 += f * ((o.mode == XT_SPH_ALL_EVAL_PARTICLES) ? P[tri(1, 0)] : P[tri(l, 0)]) * den;
      pot1 += fP * pot;
      potr += fP * frc;
      pott += f * dP[tri(l, 0)] * pot;
    }
#pragma unroll
    for (int m = 1; m <= l; ++m) {
      const R f = T.fact[l * lstride + m];
      R potc, frcc, denc, pots, frcs, dens_;
      rowvals(loff + 2 * m - 1, potc, frcc, denc);
      rowvals(loff + 2 * m, pots, frcs, dens_);
      const int k = o.trig_l ? l : m;
      const R c = cm[k], s = sm[k];
      const R fP = f * P[tri(l, m)];
      const R angp = potc * c + pots * s;
      if (dens) den1 += fP * (denc * c + dens_ * s);
      pot1 += fP * angp;
      potr += fP * (frcc * c + frcs * s);
      pott += f * dP[tri(l, m)] * angp;
      potp += fP * R(m) * (-potc * s + pots * c);
    }
  }
  out[0] = den0; out[1] = den1; out[2] = pot0; out[3] = pot1;
  out[4] = potr; out[5] = pott; out[6] = potp;
}

}  // namespace xt
