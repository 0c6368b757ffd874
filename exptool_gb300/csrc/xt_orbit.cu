// Halo + disc field composition and velocity-Verlet orbit ensembles.
//
// potential.Fields.return_forces_cart (potential.py:445-497) composes
// eof.force_eval (disc) and spheresl.force_eval (halo) into Cartesian forces;
// integrate.leapfrog_integrate (integrate.py:53-190) advances one orbit with
// x += v dt + a dt^2/2, v += (a_old + a_new) dt/2.  Here one thread owns one
// orbit for a chunk of steps: the frozen fields (coefficient-contracted tables,
// a few tens of MB) stay L2-resident, the orbit state stays in registers, and
// the kick/drift arithmetic is FP64 whatever precision the forces use.
#include <type_traits>

#include "xt_internal.cuh"
#include "xt_launch.cuh"

namespace xt {

}  // namespace xt

using namespace xt;

extern "C" {

int xt_fields_forces(void* sph, const void* sph_field, void* cyl, const void* cyl_field, int precision, int halo_l,
                     int disk_m, int no_odd, int trig_l, const double* x, const double* y, const double* z,
                     const double* rotpos, double rotpos_scalar, long long n, double* const* outs, void* stream) {
  SphTab<double> sd; SphTab<float> sf; CylTab<double> cd; CylTab<float> cf;
  XT_REQUIRE(sph_tabs(sph, &sd, &sf) && cyl_tabs(cyl, &cd, &cf), "NULL table handle");
  XT_REQUIRE(sph_field && cyl_field && outs, "NULL field or output list");
  XT_REQUIRE(n >= 0 && (n == 0 || (x && y && z)), "bad point arrays");
  XT_REQUIRE(precision == XT_F64 || precision == XT_F32, "bad precision %d", precision);
  if (n == 0) return XT_OK;
  if (halo_l < 0 || halo_l > sd.lmax) halo_l = sd.lmax;
  if (disk_m < 0 || disk_m > cd.mmax) disk_m = cd.mmax;
  FieldOpts fo{halo_l, disk_m, no_odd, trig_l, 6};
  cudaStream_t st = as_stream(stream);
  const int grid = grid_for(n, 128, 8);
  int rc = with_lcap(sd.lmax, [&](auto lc) {
    constexpr int LC = decltype(lc)::value;
    if (precision == XT_F64)
      launch_fields_forces<double, LC>(sd, static_cast<const double*>(sph_field), cd,
                                       static_cast<const double*>(cyl_field), fo, x, y, z, rotpos, rotpos_scalar, n,
                                       outs, grid, 128, st);
    else
      launch_fields_forces<float, LC>(sf, static_cast<const float*>(sph_field), cf,
                                      static_cast<const float*>(cyl_field), fo, x, y, z, rotpos, rotpos_scalar, n,
                                      outs, grid, 128, st);
    return XT_OK;
  });
  if (rc) return rc;
  XT_CHECK_LAUNCH("k_fields_forces");
  return XT_OK;
}

int xt_leapfrog(void* sph, const void* sph_field, void* cyl, const void* cyl_field, int precision, int halo_l,
                int disk_m, int no_odd, int trig_l, double* const* state, long long n, int step0, int nsteps,
                int nint, double dt, double rotc, int apse, int ap_max, double* traj, const double* dts,
                void* stream) {
  SphTab<double> sd; SphTab<float> sf; CylTab<double> cd; CylTab<float> cf;
  XT_REQUIRE(sph_tabs(sph, &sd, &sf) && cyl_tabs(cyl, &cd, &cf), "NULL table handle");
  XT_REQUIRE(sph_field && cyl_field && state, "NULL field or state");
  XT_REQUIRE(n >= 0 && step0 >= 0 && nsteps >= 0 && nint >= 1, "bad orbit counts");
  XT_REQUIRE(precision == XT_F64 || precision == XT_F32, "bad precision %d", precision);
  for (int k = 0; k < S_COUNT; ++k) XT_REQUIRE(n == 0 || state[k], "NULL state array %d", k);
  if (n == 0) return XT_OK;
  if (halo_l < 0 || halo_l > sd.lmax) halo_l = sd.lmax;
  if (disk_m < 0 || disk_m > cd.mmax) disk_m = cd.mmax;
  FieldOpts fo{halo_l, disk_m, no_odd, trig_l, 6};
  OrbitArgs A;
  for (int k = 0; k < S_COUNT; ++k) A.s[k] = state[k];
  A.n = n; A.step0 = step0; A.nsteps = nsteps; A.nint = nint; A.apse = apse; A.ap_max = ap_max;
  A.dt = dt; A.rotc = rotc; A.traj = traj; A.dts = dts;
  cudaStream_t st = as_stream(stream);
  const int grid = grid_for(n, 128, 8);
  int rc = with_lcap(sd.lmax, [&](auto lc) {
    constexpr int LC = decltype(lc)::value;
    if (precision == XT_F64)
      launch_leapfrog<double, LC>(sd, static_cast<const double*>(sph_field), cd,
                                  static_cast<const double*>(cyl_field), fo, A, grid, 128, st);
    else
      launch_leapfrog<float, LC>(sf, static_cast<const float*>(sph_field), cf, static_cast<const float*>(cyl_field),
                                 fo, A, grid, 128, st);
    return XT_OK;
  });
  if (rc) return rc;
  XT_CHECK_LAUNCH("k_leapfrog");
  return XT_OK;
}

}  // extern "C"
