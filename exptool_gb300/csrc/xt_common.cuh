// Shared host/device helpers of the exptool_gb300 CUDA library.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string>

#include "../../include/exptool_gb300.h"

namespace xt {


// ------------------------------------------------------------------ errors
void set_error(const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

#define XT_CUDA(call)                                              \
  do {                                                             \
    cudaError_t _e = (call);                                       \
    if (_e != cudaSuccess) return ::xt::cuda_fail(_e, #call);      \
  } while (0)

#define XT_CHECK_LAUNCH(what)                                      \
  do {                                                             \
    cudaError_t _e = cudaGetLastError();                           \
    if (_e != cudaSuccess) return ::xt::cuda_fail(_e, what);       \
  } while (0)

#define XT_REQUIRE(cond, ...)                                      \
  do {                                                             \
    if (!(cond)) {                                                 \
      ::xt::set_error(__VA_ARGS__);                                \
      return XT_ERR_ARG;                                           \
    }                                                              \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Grid size for a grid-stride loop over n items: a multiple of the SM count
// (152 on GB300) times the resident blocks per SM, capped by the work.
int grid_for(long long n, int block, int blocks_per_sm = 8);
int sm_count();   // multiprocessors of the current device (cached)

// Blocks of `fn` (a __global__ function) resident per SM at this block size and
// dynamic shared memory (cudaOccupancyMaxActiveBlocksPerMultiprocessor, cached).
int resident_blocks_per_sm(const void* fn, int block, size_t smem);

// For a kernel with large dynamic shared memory: asks for the whole unified
// L1/shared storage as shared memory (carveout 100) and returns the blocks
// resident per SM under that carveout.  The occupancy API counts shared memory
// against the default carveout, not the preference, so the shared-memory limit
// is computed here from the SM's shared memory, the per-block reservation and
// the 128-byte allocation granularity; registers, warps and the block limit
// come from the occupancy API without dynamic shared memory.  Returns 0 when a
// block does not fit.
int resident_blocks_full_carveout(const void* fn, int block, size_t smem);

// Blocks of a kernel that allocates `tmem_cols` tensor-memory columns per
// block, resident per SM, from the SM's own limits: registers (per-thread
// count rounded to 8, per warp to 256), threads, blocks, shared memory under
// the full carveout (as above) and the 512 tensor-memory columns.  The
// occupancy API answers 1 for kernels that contain tcgen05.alloc whatever
// their resources (measured on GB300: four 128-thread CTAs of 49 KB run
// together and take 6.4 ms where one per SM takes 12.3 ms), so it is not
// asked.  Returns 0 when a block does not fit.
int resident_blocks_tmem(const void* fn, int block, size_t smem, int tmem_cols);

// Grid of at most one full wave: as many blocks as stay resident together, or
// fewer when `units` (one per thread) needs fewer.  Grid-stride kernels launched
// this way balance their work over every resident block instead of leaving a
// partial last wave.
template <typename Kern>
int resident_grid(Kern fn, int block, size_t smem, long long units) {
  const long long cap = (long long)resident_blocks_per_sm((const void*)fn, block, smem) * sm_count();
  long long need = (units + block - 1) / block;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

// Where a pointer lives, as far as kernels are concerned (XT_PTR_* values of
// the public header): device (or managed) memory, pinned host memory, other
// host memory the device can address (pageable access), or host memory it
// cannot address.
int pointer_access(const void* p);

// ------------------------------------------------------------------ device math
constexpr double PI = 3.14159265358979323846;

template <typename R>
__device__ __forceinline__ bool finite(R v) { return isfinite(v); }

// compatibility.r_to_xi (exptool/basis/compatibility.py:16-49): r < 0 maps to 0.
template <typename R>
__device__ __forceinline__ R r_to_xi(R r, int cmap, R scale) {
  R out;
  if (cmap == 1) {
    out = (r / scale - R(1)) / (r / scale + R(1));
  } else if (cmap == 2) {
    out = log(r);
  } else {
    out = r;
  }
  return (r < R(0)) ? R(0) : out;
}

// r_to_xi with the scale division replaced by a multiplication by its
// reciprocal (one rounding of difference; FP64 division is a multi-instruction
// sequence on the FP64 pipe).
template <typename R>
__device__ __forceinline__ R r_to_xi_inv(R r, int cmap, R inv_scale) {
  R out;
  if (cmap == 1) {
    const R u = r * inv_scale;
    out = (u - R(1)) / (u + R(1));
  } else if (cmap == 2) {
    out = log(r);
  } else {
    out = r;
  }
  return (r < R(0)) ? R(0) : out;
}

// compatibility.d_xi_to_r (compatibility.py:65-80)
template <typename R>
__device__ __forceinline__ R d_xi_to_r(R xi, int cmap, R scale) {
  if (cmap == 1) return R(0.5) * (R(1) - xi) * (R(1) - xi) / scale;
  if (cmap == 2) return exp(-xi);
  return R(1);
}

// compatibility.z_to_y (compatibility.py:83-91): z/(|z|+1e-8) * asinh(|z/h|)
template <typename R>
__device__ __forceinline__ R z_to_y(R z, R hscale) {
  return (z / (fabs(z) + R(1.0e-8))) * asinh(fabs(z / hscale));
}

// z_to_y with z/h as a multiplication by 1/h.
template <typename R>
__device__ __forceinline__ R z_to_y_inv(R z, R inv_hscale) {
  return (z / (fabs(z) + R(1.0e-8))) * asinh(fabs(z * inv_hscale));
}

// cos(phi), sin(phi) of phi = atan2(y, x) without the arctangent:
// x/rho, y/rho; rho == 0 keeps atan2's signed-zero conventions.
template <typename R>
__device__ __forceinline__ void unit_phi(R x, R y, R& c, R& s) {
  R rho = sqrt(x * x + y * y);
  if (rho > R(0)) {
    R inv = R(1) / rho;
    c = x * inv;
    s = y * inv;
  } else {
    R p = atan2(y, x);
    c = cos(p);
    s = sin(p);
  }
}

template <typename R>
__device__ __forceinline__ void sincos_r(R a, R* s, R* c);
template <>
__device__ __forceinline__ void sincos_r<double>(double a, double* s, double* c) { sincos(a, s, c); }
template <>
__device__ __forceinline__ void sincos_r<float>(float a, float* s, float* c) { sincosf(a, s, c); }

}  // namespace xt
