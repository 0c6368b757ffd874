// Launcher declarations shared between the ABI files and the per-precision
// kernel translation units (xt_*_k64.cu, xt_*_k32.cu), plus the lmax dispatch.
#pragma once

#include <type_traits>

#include "xt_internal.cuh"

namespace xt {

struct FieldOpts {
  int halo_l, disk_m, no_odd, trig_l, nf;
};

// Orbit state slots (structure of arrays, each n doubles).
enum { S_X, S_Y, S_Z, S_VX, S_VY, S_VZ, S_FX, S_FY, S_FZ, S_POT, S_R2M1, S_R2M2, S_APS, S_NSTEP, S_E0, S_EDEV, S_COUNT };

struct OrbitArgs {
  double* s[S_COUNT];
  long long n;
  int step0, nsteps, nint, apse, ap_max;
  double dt, rotc;
  double* traj;
  const double* dts;          // per-orbit step sizes (NULL: dt for all)
};

template <typename R, int LC>
void launch_sph_deposit(const SphTab<R>& T, const double* x, const double* y, const double* z, const double* m,
                        long long n, int no_odd, double* D, int grid, int block, cudaStream_t st);
template <typename R, int LC>
void launch_sph_eval(const SphTab<R>& T, const R* GH, int coord_mode, const double* a, const double* b,
                     const double* c, long long n, const SphEvalOpts& o, double* const* outs, int grid, int block,
                     cudaStream_t st);
template <typename R, int LC>
void launch_fields_forces(const SphTab<R>& ST, const R* GH, const CylTab<R>& CT, const R* F, const FieldOpts& fo,
                          const double* x, const double* y, const double* z, const double* rot, double rot_scalar,
                          long long n, double* const* outs, int grid, int block, cudaStream_t st);
template <typename R, int LC>
void launch_leapfrog(const SphTab<R>& ST, const R* GH, const CylTab<R>& CT, const R* F, const FieldOpts& fo,
                     const OrbitArgs& A, int grid, int block, cudaStream_t st);

// Compile-time lmax capacity: fully unrolled, register-resident Legendre and
// trigonometric tables for lmax <= 4, 6 and 8.
template <typename F>
inline int with_lcap(int lmax, F&& f) {
  if (lmax <= 4) return f(std::integral_constant<int, 4>{});
  if (lmax <= 6) return f(std::integral_constant<int, 6>{});
  if (lmax <= 8) return f(std::integral_constant<int, 8>{});
  set_error("lmax %d exceeds the supported maximum 8", lmax);
  return XT_ERR_ARG;
}

}  // namespace xt
