// Field-composition and leapfrog kernels with their launchers; instantiated
// per precision in xt_orbit_k64.cu / xt_orbit_k32.cu.
#pragma once

#include <type_traits>

#include "xt_df.cuh"
#include "xt_launch.cuh"

namespace xt {

// Exact widening of a force component to FP64: for FP32 forces by integer
// operations (the same double as the conversion instruction, without the
// FP64 pipe, which the FP64 kick/drift of the orbit step keeps busy).
__device__ __forceinline__ double wide(float v) { return f2d_int(v); }
__device__ __forceinline__ double wide(double v) { return v; }

// One point of Fields.return_forces_cart: out = fxd fxh fyd fyh fzd fzh diskp halop.
// (cr, sr) = cos/sin of the rotation angle added to phi.
template <typename R, int LCAP>
__device__ __forceinline__ void fields_point(const SphTab<R>& ST, const R* __restrict__ GH, const CylTab<R>& CT,
                                             const R* __restrict__ F, const FieldOpts& fo, R x, R y, R z, R cr,
                                             R sr, R out[8]) {
  const R r2 = sqrt(x * x + y * y) + R(1.0e-15);
  const R r3 = sqrt(r2 * r2 + z * z) + R(1.0e-15);
  const R costh = z / r3;
  R cp, sp;
  unit_phi(x, y, cp, sp);
  const R c1 = cp * cr - sp * sr;   // cos(phi + rotpos)
  const R s1 = sp * cr + cp * sr;   // sin(phi + rotpos)
  CylEvalOpts co;
  co.mode = XT_CYL_FORCE_EVAL; co.m1 = 0; co.m2 = 1 << 30; co.mmax_use = fo.disk_m; co.no_odd = fo.no_odd;
  co.perturb = 0; co.density = 0; co.nf = fo.nf;
  R dv[9];
  cyl_eval_point<R, 16>(CT, F, r2, z, c1, s1, co, dv);
  R diskfr = dv[2] + dv[7], diskfp = dv[3], diskfz = dv[4] + dv[8], diskp = dv[1] + dv[0];
  SphEvalOpts so;
  so.mode = XT_SPH_FORCE_EVAL; so.L1 = -1000; so.L2 = 1000; so.no_odd = fo.no_odd; so.lmax_use = fo.halo_l;
  so.trig_l = fo.trig_l; so.want_dens = 0;
  R hv[7];
  sph_eval_point<R, LCAP>(ST, GH, r3, costh, c1, s1, so, hv);
  const R halofr = hv[4], haloft = hv[5];
  R halofp = hv[6];
  const R halop = hv[3] + hv[2];
  if (r3 < ST.xi0) {        // potential.py:481-483 guard against r < min(xi)
    halofp = R(0);
    diskfp = R(0);
  }
  const R r22 = r2 * r2, r33 = r3 * r3 * r3;
  out[0] = diskfr * (x / r2) - diskfp * (y / r22);
  out[1] = -(halofr * (x / r3) - haloft * (x * z / r33)) + halofp * (y / r22);
  out[2] = diskfr * (y / r2) + diskfp * (x / r22);
  out[3] = -(halofr * (y / r3) - haloft * (y * z / r33)) - halofp * (x / r22);
  out[4] = diskfz;
  out[5] = -(halofr * (z / r3) + haloft * (r22 / r33));
  out[6] = diskp;
  out[7] = halop;
}

template <typename R, int LCAP>
__global__ void __launch_bounds__(128) k_fields_forces(SphTab<R> ST, const R* __restrict__ GH, CylTab<R> CT,
                                                       const R* __restrict__ F, FieldOpts fo,
                                                       const double* __restrict__ x, const double* __restrict__ y,
                                                       const double* __restrict__ z, const double* __restrict__ rot,
                                                       double rot_scalar, long long n, double* o0, double* o1,
                                                       double* o2, double* o3, double* o4, double* o5, double* o6,
                                                       double* o7) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const double rp = rot ? rot[p] : rot_scalar;
    double srd, crd;
    sincos(rp, &srd, &crd);
    R v[8];
    fields_point<R, LCAP>(ST, GH, CT, F, fo, (R)x[p], (R)y[p], (R)z[p], (R)crd, (R)srd, v);
    double* outs[8] = {o0, o1, o2, o3, o4, o5, o6, o7};
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (outs[k]) outs[k][p] = (double)v[k];
  }
}

__device__ __forceinline__ void traj_row(double* traj, long long p, int nint, int k, const double* q) {
  double* t = traj + ((size_t)p * nint + k) * 10;
#pragma unroll
  for (int i = 0; i < 10; ++i) t[i] = q[i];
}

// One orbit of the FP32-force leapfrog with its state (position, velocity,
// forces, potential, squared radii, energies) in double-float on the FP32
// pipe: GB300 issues two FP64 FMAs per clock per SM against 128 FP32, and the
// FP64 kick/drift of about 50 FP64 operations per step bound the FP32-force
// step.  The same steps as the FP64 state below (integrate.py:116-160), with
// sums of the two FP32 force parts exact (TwoSum) and positions rounded to
// FP32 for the force evaluation.  The state is read and written as FP64
// (split and widened by integer operations).
template <int LCAP>
__device__ __forceinline__ void leapfrog_orbit_df(const SphTab<float>& ST, const float* __restrict__ GH,
                                                  const CylTab<float>& CT, const float* __restrict__ F,
                                                  const FieldOpts& fo, const OrbitArgs& A, long long p) {
  df x = df_split_or_from(A.s[S_X][p]), y = df_split_or_from(A.s[S_Y][p]), z = df_split_or_from(A.s[S_Z][p]);
  df vx = df_split_or_from(A.s[S_VX][p]), vy = df_split_or_from(A.s[S_VY][p]),
     vz = df_split_or_from(A.s[S_VZ][p]);
  df fx, fy, fz, pot, r2m1, r2m2, e0, edev;
  float aps;
  int nstep;
  float v[8];
  auto posf = [](df a) { return __fadd_rn(a.h, a.l); };
  auto energy = [&]() {
    const df k2 = df_add(df_add(df_mul(vx, vx), df_mul(vy, vy)), df_mul(vz, vz));
    return df_add(df{0.5f * k2.h, 0.5f * k2.l}, pot);
  };
  auto row = [&](int k) {
    const double q[10] = {df_to_int(x),  df_to_int(y),   df_to_int(z),  df_to_int(vx), df_to_int(vy),
                          df_to_int(vz), df_to_int(pot), df_to_int(fx), df_to_int(fy), df_to_int(fz)};
    traj_row(A.traj, p, A.nint, k, q);
  };
  if (A.step0 == 0) {
    fields_point<float, LCAP>(ST, GH, CT, F, fo, posf(x), posf(y), posf(z), 1.f, 0.f, v);
    fx = df_two_sum(v[0], v[1]);
    fy = df_two_sum(v[2], v[3]);
    fz = df_two_sum(v[4], v[5]);
    pot = df_two_sum(v[6], v[7]);
    r2m1 = df_add(df_mul(x, x), df_mul(y, y));
    r2m2 = {0.f, 0.f};
    aps = 0.f;
    nstep = 1;
    e0 = energy();
    edev = {0.f, 0.f};
    if (A.traj) row(0);
  } else {
    fx = df_split_or_from(A.s[S_FX][p]);
    fy = df_split_or_from(A.s[S_FY][p]);
    fz = df_split_or_from(A.s[S_FZ][p]);
    pot = df_split_or_from(A.s[S_POT][p]);
    r2m1 = df_split_or_from(A.s[S_R2M1][p]);
    r2m2 = df_split_or_from(A.s[S_R2M2][p]);
    aps = (float)A.s[S_APS][p];
    nstep = (int)A.s[S_NSTEP][p];
    e0 = df_split_or_from(A.s[S_E0][p]);
    edev = df_split_or_from(A.s[S_EDEV][p]);
  }
  const double dtv = A.dts ? A.dts[p] : A.dt;
  const df dt = df_split_or_from(dtv), hdt = {0.5f * dt.h, 0.5f * dt.l};
  const df hdt2 = df_mul(hdt, dt);   // dt^2 / 2
  const float apmax = (float)A.ap_max;
  const int kbeg = A.step0 < 1 ? 1 : A.step0;
  int kend = A.step0 + A.nsteps;
  if (kend > A.nint) kend = A.nint;
  for (int k = kbeg; k < kend; ++k) {
    if (!(aps < apmax)) break;   // integrate.py:126 loop condition
    if (nstep != k) break;       // orbit already stopped
    x = df_add(df_add(x, df_mul(vx, dt)), df_mul(fx, hdt2));
    y = df_add(df_add(y, df_mul(vy, dt)), df_mul(fy, hdt2));
    z = df_add(df_add(z, df_mul(vz, dt)), df_mul(fz, hdt2));
    float srd = 0.f, crd = 1.f;
    if (A.rotc != 0.0) {
      double sd, cd;
      sincos(A.rotc * ((double)k * dtv), &sd, &cd);
      srd = (float)sd;
      crd = (float)cd;
    }
    fields_point<float, LCAP>(ST, GH, CT, F, fo, posf(x), posf(y), posf(z), crd, srd, v);
    const df nfx = df_two_sum(v[0], v[1]), nfy = df_two_sum(v[2], v[3]), nfz = df_two_sum(v[4], v[5]);
    pot = df_two_sum(v[6], v[7]);
    vx = df_add(vx, df_mul(df_add(fx, nfx), hdt));
    vy = df_add(vy, df_mul(df_add(fy, nfy), hdt));
    vz = df_add(vz, df_mul(df_add(fz, nfz), hdt));
    fx = nfx;
    fy = nfy;
    fz = nfz;
    const df r2now = df_add(df_mul(x, x), df_mul(y, y));
    if (A.apse && k > 1 && df_gt(r2m1, r2m2) && df_gt(r2m1, r2now)) aps += 1.f;
    r2m2 = r2m1;
    r2m1 = r2now;
    nstep = k + 1;
    df de = df_sub(energy(), e0);
    if (de.h < 0.f) de = df_neg(de);
    if (df_gt(de, edev)) edev = de;
    if (A.traj) row(k);
  }
  A.s[S_X][p] = df_to_int(x); A.s[S_Y][p] = df_to_int(y); A.s[S_Z][p] = df_to_int(z);
  A.s[S_VX][p] = df_to_int(vx); A.s[S_VY][p] = df_to_int(vy); A.s[S_VZ][p] = df_to_int(vz);
  A.s[S_FX][p] = df_to_int(fx); A.s[S_FY][p] = df_to_int(fy); A.s[S_FZ][p] = df_to_int(fz);
  A.s[S_POT][p] = df_to_int(pot);
  A.s[S_R2M1][p] = df_to_int(r2m1); A.s[S_R2M2][p] = df_to_int(r2m2);
  A.s[S_APS][p] = (double)aps;
  A.s[S_NSTEP][p] = (double)nstep;
  A.s[S_E0][p] = df_to_int(e0); A.s[S_EDEV][p] = df_to_int(edev);
}

template <typename R, int LCAP>
__global__ void __launch_bounds__(128, 4) k_leapfrog(SphTab<R> ST, const R* __restrict__ GH, CylTab<R> CT,
                                                  const R* __restrict__ F, FieldOpts fo, OrbitArgs A) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < A.n;
       p += (long long)gridDim.x * blockDim.x) {
    if constexpr (std::is_same<R, float>::value) {
      leapfrog_orbit_df<LCAP>(ST, GH, CT, F, fo, A, p);
      continue;
    }
    double x = A.s[S_X][p], y = A.s[S_Y][p], z = A.s[S_Z][p];
    double vx = A.s[S_VX][p], vy = A.s[S_VY][p], vz = A.s[S_VZ][p];
    double fx, fy, fz, pot, r2m1, r2m2, aps, e0, edev;
    int nstep;
    R v[8];
    if (A.step0 == 0) {
      // integrate.py:116-122: forces at the initial position, rotation 0
      fields_point<R, LCAP>(ST, GH, CT, F, fo, (R)x, (R)y, (R)z, R(1), R(0), v);
      fx = wide(v[0]) + wide(v[1]);
      fy = wide(v[2]) + wide(v[3]);
      fz = wide(v[4]) + wide(v[5]);
      pot = wide(v[6]) + wide(v[7]);
      r2m1 = x * x + y * y;
      r2m2 = 0.0;
      aps = 0.0;
      nstep = 1;
      e0 = 0.5 * (vx * vx + vy * vy + vz * vz) + pot;
      edev = 0.0;
      if (A.traj) {
        const double q[10] = {x, y, z, vx, vy, vz, pot, fx, fy, fz};
        traj_row(A.traj, p, A.nint, 0, q);
      }
    } else {
      fx = A.s[S_FX][p]; fy = A.s[S_FY][p]; fz = A.s[S_FZ][p]; pot = A.s[S_POT][p];
      r2m1 = A.s[S_R2M1][p]; r2m2 = A.s[S_R2M2][p]; aps = A.s[S_APS][p];
      nstep = (int)A.s[S_NSTEP][p]; e0 = A.s[S_E0][p]; edev = A.s[S_EDEV][p];
    }
    const double dt = A.dts ? A.dts[p] : A.dt, dt2 = dt * dt;
    const int kbeg = A.step0 < 1 ? 1 : A.step0;
    int kend = A.step0 + A.nsteps;
    if (kend > A.nint) kend = A.nint;
    for (int k = kbeg; k < kend; ++k) {
      if (!(aps < (double)A.ap_max)) break;   // integrate.py:126 loop condition
      if (nstep != k) break;                   // orbit already stopped
      x = x + (vx * dt) + (0.5 * fx * dt2);
      y = y + (vy * dt) + (0.5 * fy * dt2);
      z = z + (vz * dt) + (0.5 * fz * dt2);
      // rotation of the field frame (integrate.py:131); without rotation the
      // angle is zero at every step and its FP64 sine and cosine are skipped
      double srd = 0.0, crd = 1.0;
      if (A.rotc != 0.0) sincos(A.rotc * ((double)k * dt), &srd, &crd);
      fields_point<R, LCAP>(ST, GH, CT, F, fo, (R)x, (R)y, (R)z, (R)crd, (R)srd, v);
      const double nfx = wide(v[0]) + wide(v[1]);
      const double nfy = wide(v[2]) + wide(v[3]);
      const double nfz = wide(v[4]) + wide(v[5]);
      pot = wide(v[6]) + wide(v[7]);
      vx = vx + (0.5 * (fx + nfx) * dt);
      vy = vy + (0.5 * (fy + nfy) * dt);
      vz = vz + (0.5 * (fz + nfz) * dt);
      fx = nfx; fy = nfy; fz = nfz;
      const double r2now = x * x + y * y;
      if (A.apse && k > 1 && (r2m1 > r2m2) && (r2m1 > r2now)) aps += 1.0;
      r2m2 = r2m1;
      r2m1 = r2now;
      nstep = k + 1;
      const double e = 0.5 * (vx * vx + vy * vy + vz * vz) + pot;
      const double de = fabs(e - e0);
      edev = de > edev ? de : edev;
      if (A.traj) {
        const double q[10] = {x, y, z, vx, vy, vz, pot, fx, fy, fz};
        traj_row(A.traj, p, A.nint, k, q);
      }
    }
    A.s[S_X][p] = x; A.s[S_Y][p] = y; A.s[S_Z][p] = z;
    A.s[S_VX][p] = vx; A.s[S_VY][p] = vy; A.s[S_VZ][p] = vz;
    A.s[S_FX][p] = fx; A.s[S_FY][p] = fy; A.s[S_FZ][p] = fz; A.s[S_POT][p] = pot;
    A.s[S_R2M1][p] = r2m1; A.s[S_R2M2][p] = r2m2; A.s[S_APS][p] = aps;
    A.s[S_NSTEP][p] = (double)nstep; A.s[S_E0][p] = e0; A.s[S_EDEV][p] = edev;
  }
}

template <typename R, int LC>
void launch_fields_forces(const SphTab<R>& ST, const R* GH, const CylTab<R>& CT, const R* F, const FieldOpts& fo,
                          const double* x, const double* y, const double* z, const double* rot, double rot_scalar,
                          long long n, double* const* outs, int grid, int block, cudaStream_t st) {
  k_fields_forces<R, LC><<<grid, block, 0, st>>>(ST, GH, CT, F, fo, x, y, z, rot, rot_scalar, n, outs[0], outs[1],
                                                 outs[2], outs[3], outs[4], outs[5], outs[6], outs[7]);
}

template <typename R, int LC>
void launch_leapfrog(const SphTab<R>& ST, const R* GH, const CylTab<R>& CT, const R* F, const FieldOpts& fo,
                     const OrbitArgs& A, int grid, int block, cudaStream_t st) {
  k_leapfrog<R, LC><<<grid, block, 0, st>>>(ST, GH, CT, F, fo, A);
}

}  // namespace xt
