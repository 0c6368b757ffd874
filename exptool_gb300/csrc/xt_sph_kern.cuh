// Spherical per-particle kernels (deposition and evaluation) and their
// launchers; instantiated per precision in xt_sph_k64.cu / xt_sph_k32.cu so
// the heavily unrolled Legendre loops compile in parallel.
#pragma once

#include "xt_launch.cuh"

namespace xt {

constexpr double FOUR_PI = 4.0 * PI;

// One thread per particle: deposit -4 pi m plerp Y_lm(theta, phi) x {x1, x2}
// onto D[row][node] (FP64 atomics at L2).  r = max(|x|, 1e-10) with NaN -> 1e-10
// as np.nanmax (spheresl.py:611).
template <typename R, int LCAP>
__global__ void __launch_bounds__(256) k_sph_deposit(SphTab<R> T, const double* __restrict__ x,
                                                     const double* __restrict__ y, const double* __restrict__ z,
                                                     const double* __restrict__ mass, long long n, int no_odd,
                                                     double* __restrict__ D) {
  constexpr int NT = (LCAP + 1) * (LCAP + 2) / 2;
  const int lmax = T.lmax;
  const int numr = T.numr;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const R xx = (R)x[p], yy = (R)y[p], zz = (R)z[p];
    const R mm = (R)mass[p];
    R r = sqrt(xx * xx + yy * yy + zz * zz);
    if (!(r >= R(1.0e-10))) r = R(1.0e-10);
    const R costh = zz / r;
    R c1, s1;
    unit_phi(xx, yy, c1, s1);
    R P[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) P[k] = R(0);
    legendre<R, LCAP>(costh, lmax, P);
    R cm[LCAP + 1], sm[LCAP + 1];
    multiples<R, LCAP>(c1, s1, lmax, cm, sm);
    SphBins<R> B = sph_bins(T, r, false, false);
    const int i0 = B.i;
    R w0 = B.lw0, w1 = B.lw1;
    const R base = R(-FOUR_PI) * mm;
    w0 *= base;
    w1 *= base;
    const int lstride = lmax + 1;
#pragma unroll
    for (int l = 0; l <= LCAP; ++l) {
      if (l > lmax) break;
      if (no_odd && (l & 1)) continue;
      const int loff = l * l;
#pragma unroll
      for (int m = 0; m <= l; ++m) {
        const R a = T.fact[l * lstride + m] * P[tri(l, m)];
        if (m == 0) {
          double* d = D + (size_t)loff * numr + i0;
          atomicAdd(d, (double)(a * w0));
          atomicAdd(d + 1, (double)(a * w1));
        } else {
          const R ac = a * cm[m], as = a * sm[m];
          double* dc = D + (size_t)(loff + 2 * m - 1) * numr + i0;
          double* ds = dc + numr;
          atomicAdd(dc, (double)(ac * w0));
          atomicAdd(dc + 1, (double)(ac * w1));
          atomicAdd(ds, (double)(as * w0));
          atomicAdd(ds + 1, (double)(as * w1));
        }
      }
    }
  }
}

template <typename R, int LCAP>
__global__ void __launch_bounds__(128) k_sph_eval(SphTab<R> T, const R* __restrict__ GH, int coord_mode,
                                                  const double* __restrict__ a, const double* __restrict__ b,
                                                  const double* __restrict__ c, long long n, SphEvalOpts o,
                                                  double* o0, double* o1, double* o2, double* o3, double* o4,
                                                  double* o5, double* o6, double* o7) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    R r, costh, c1, s1, rr = R(0);
    if (coord_mode == XT_COORD_CART) {
      const R xx = (R)a[p], yy = (R)b[p], zz = (R)c[p];
      r = sqrt(xx * xx + yy * yy + zz * zz);
      rr = sqrt(xx * xx + yy * yy);
      costh = zz / r;
      unit_phi(xx, yy, c1, s1);
    } else {
      r = (R)a[p];
      costh = (R)b[p];
      sincos_r((R)c[p], &s1, &c1);
    }
    R v[7];
    sph_eval_point<R, LCAP>(T, GH, r, costh, c1, s1, o, v);
    if (o.mode == XT_SPH_FORCE_EVAL) {
      // potr pott potp pot1 pot0
      if (o0) o0[p] = (double)v[4];
      if (o1) o1[p] = (double)v[5];
      if (o2) o2[p] = (double)v[6];
      if (o3) o3[p] = (double)v[3];
      if (o4) o4[p] = (double)v[2];
    } else {
      const double densfac = (o.mode == XT_SPH_ALL_EVAL_PARTICLES) ? 0.25 * PI : 0.25 / PI;
      if (o0) o0[p] = (double)v[0] * densfac;
      if (o1) o1[p] = (double)v[1] * densfac;
      if (o2) o2[p] = (double)v[2];
      if (o3) o3[p] = (double)v[3];
      if (o4) o4[p] = (double)v[4];
      if (o5) o5[p] = (double)v[5];
      if (o6) o6[p] = (double)v[6];
      if (o7 && o.mode == XT_SPH_ALL_EVAL_PARTICLES) o7[p] = (double)rr;
    }
  }
}



template <typename R, int LC>
void launch_sph_deposit(const SphTab<R>& T, const double* x, const double* y, const double* z, const double* m,
                        long long n, int no_odd, double* D, int grid, int block, cudaStream_t st) {
  k_sph_deposit<R, LC><<<grid, block, 0, st>>>(T, x, y, z, m, n, no_odd, D);
}

template <typename R, int LC>
void launch_sph_eval(const SphTab<R>& T, const R* GH, int coord_mode, const double* a, const double* b,
                     const double* c, long long n, const SphEvalOpts& o, double* const* outs, int grid, int block,
                     cudaStream_t st) {
  k_sph_eval<R, LC><<<grid, block, 0, st>>>(T, GH, coord_mode, a, b, c, n, o, outs[0], outs[1], outs[2], outs[3],
                                            outs[4], outs[5], outs[6], outs[7]);
}

}  // namespace xt
