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

// ---------------------------------------------------------------- orbit reordering
// Ensembles of orbits at unrelated positions make every warp gather its
// field values from unrelated table cells.  Between chunks of steps the
// orbits are counting-sorted by the disc table cell of their position
// (eof.return_bins's cell, eof.py:354-427, from FP32 coordinates), so that the
// threads of a warp share cells and their gathers hit L1.  The state moves
// with its orbit (16 rows of n doubles) together with the orbit's original
// index; each orbit's arithmetic is unchanged, so results are bit-identical
// to the unsorted run once xt_orbit_unsort restores the order.
__global__ void __launch_bounds__(256) k_orbit_key(CylTab<float> T, const double* __restrict__ s, long long n,
                                                   int* __restrict__ hist, int* __restrict__ key,
                                                   int* __restrict__ slot) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float x = (float)s[S_X * n + q], y = (float)s[S_Y * n + q], z = (float)s[S_Z * n + q];
    const CylBins<float> B = cyl_bins(T, sqrtf(x * x + y * y), z);
    const int ix = B.node / (T.numy + 1), iy = B.node - ix * (T.numy + 1);
    const int cell = ix * T.numy + iy;
    key[q] = cell;
    slot[q] = atomicAdd(hist + cell, 1);
  }
}

__global__ void __launch_bounds__(256) k_orbit_gather(const double* __restrict__ in, double* __restrict__ out,
                                                      long long n, const int* __restrict__ off,
                                                      const int* __restrict__ key, const int* __restrict__ slot,
                                                      const long long* __restrict__ order_in,
                                                      long long* __restrict__ order_out) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const long long d = (long long)off[key[q]] + slot[q];
#pragma unroll
    for (int k = 0; k < S_COUNT; ++k) out[k * n + d] = in[k * n + q];
    order_out[d] = order_in[q];
  }
}

__global__ void __launch_bounds__(256) k_orbit_unsort(const double* __restrict__ in, double* __restrict__ out,
                                                      long long n, const long long* __restrict__ order) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const long long d = order[q];
#pragma unroll
    for (int k = 0; k < S_COUNT; ++k) out[k * n + d] = in[k * n + q];
  }
}

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

size_t xt_orbit_sort_workspace(void* cyl, long long n) {
  CylTab<double> cd;
  CylTab<float> cf;
  if (!cyl_tabs(cyl, &cd, &cf) || n < 0) return 0;
  return (2 * (size_t)cf.numx * cf.numy + 2 * (size_t)n + 1024) * sizeof(int) + 256;
}

int xt_orbit_sort(void* cyl, const double* state_in, double* state_out, long long n, const long long* order_in,
                  long long* order_out, void* workspace, size_t workspace_bytes, void* stream) {
  CylTab<double> cd;
  CylTab<float> cf;
  XT_REQUIRE(cyl_tabs(cyl, &cd, &cf), "NULL table handle");
  XT_REQUIRE(n >= 0 && n < (1LL << 31), "orbit count must be in [0, 2^31)");
  if (n == 0) return XT_OK;
  XT_REQUIRE(state_in && state_out && order_in && order_out && state_in != state_out && order_in != order_out,
             "need distinct input and output states and orders");
  const size_t need = xt_orbit_sort_workspace(cyl, n);
  if (!workspace || workspace_bytes < need) {
    set_error("workspace of %zu bytes needed, %zu given", need, workspace_bytes);
    return XT_ERR_WORKSPACE;
  }
  const int ncell = cf.numx * cf.numy;
  XT_REQUIRE(ncell >= 1 && ncell <= (1 << 20), "table of %d cells", ncell);
  int* hist = static_cast<int*>(workspace);
  int* off = hist + ncell;
  int* tsum = off + ncell;
  int* key = tsum + 1024;
  int* slot = key + n;
  cudaStream_t st = as_stream(stream);
  XT_CUDA(cudaMemsetAsync(hist, 0, (size_t)ncell * sizeof(int), st));
  const int grid = grid_for(n, 256, 8);
  k_orbit_key<<<grid, 256, 0, st>>>(cf, state_in, n, hist, key, slot);
  XT_CHECK_LAUNCH("k_orbit_key");
  int rc = launch_cell_scan(hist, off, tsum, ncell, st);
  if (rc) return rc;
  k_orbit_gather<<<grid, 256, 0, st>>>(state_in, state_out, n, off, key, slot, order_in, order_out);
  XT_CHECK_LAUNCH("k_orbit_gather");
  return XT_OK;
}

int xt_orbit_unsort(const double* state_in, double* state_out, long long n, const long long* order, void* stream) {
  XT_REQUIRE(n >= 0 && n < (1LL << 31), "orbit count must be in [0, 2^31)");
  if (n == 0) return XT_OK;
  XT_REQUIRE(state_in && state_out && order && state_in != state_out, "need distinct states and an order");
  k_orbit_unsort<<<grid_for(n, 256, 8), 256, 0, as_stream(stream)>>>(state_in, state_out, n, order);
  XT_CHECK_LAUNCH("k_orbit_unsort");
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
