// Spherical SL basis: table upload, coefficient accumulation, evaluation.
//
// Accumulation (spheresl.compute_coefficients_solitary, spheresl.py:567-656)
// is restructured for GB300, whose FP64 pipe runs at a small fraction of its
// FP32 rate: instead of forming all (lmax+1)^2 x nmax products per particle,
// each particle deposits its angular weight
//     A_row = -4 pi * mass * plerp * fact[l][m] * P_l^m(cos th) * {1, cos m phi, sin m phi}
// onto the two radial nodes it interpolates between (weights x1, x2), and one
// memory-bound pass contracts the node grid with ef/sqrt(ev):
//     expcoef[row, n] = sum_i ef[l,n,i]/sqrt(ev[l,n]) * D[row, i]
// which is the reference sum reordered (the potential lerp is linear in ef).
// Evaluation first contracts the coefficients with the radial tables (per
// node, per row) so each point does 3-point gathers per row instead of
// nmax-long dot products.
#include <cuda.h>

#include <algorithm>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "xt_internal.cuh"
#include "xt_launch.cuh"

namespace xt {

// ------------------------------------------------------------------ error state
static thread_local std::string g_err;

void set_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}

int cuda_fail(cudaError_t e, const char* what) {
  set_error("CUDA error %s (%d) in %s", cudaGetErrorString(e), (int)e, what);
  return (e == cudaErrorMemoryAllocation) ? XT_ERR_OOM : XT_ERR_CUDA;
}

int sm_count() {
  static int nsm = 0;
  if (nsm == 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    nsm = (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0) ? v : 152;
  }
  return nsm;
}

int resident_blocks_per_sm(const void* fn, int block, size_t smem) {
  struct Key {
    const void* fn;
    int block;
    size_t smem;
  };
  static std::mutex mu;
  static std::vector<std::pair<Key, int>> cache;
  std::lock_guard<std::mutex> lock(mu);
  for (const auto& e : cache)
    if (e.first.fn == fn && e.first.block == block && e.first.smem == smem) return e.second;
  int v = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, fn, block, smem) != cudaSuccess || v < 1) {
    cudaGetLastError();
    return 1;                                   // not cached: asked again next time
  }
  cache.push_back({Key{fn, block, smem}, v});
  return v;
}

int resident_blocks_full_carveout(const void* fn, int block, size_t smem) {
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int dev = 0, per_sm_smem = 0, reserved = 0, other = 0;
  cudaFuncAttributes fa{};
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&per_sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
      cudaFuncGetAttributes(&fa, fn) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&other, fn, block, 0) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  const size_t per_block = (smem + fa.sharedSizeBytes + (size_t)reserved + 127) / 128 * 128;
  const int by_smem = (int)((size_t)per_sm_smem / per_block);
  return by_smem < other ? by_smem : other;
}

int resident_blocks_tmem(const void* fn, int block, size_t smem, int tmem_cols) {
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
      cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int dev = 0, per_sm_smem = 0, reserved = 0, regs_sm = 0, threads_sm = 0, blocks_sm = 0;
  cudaFuncAttributes fa{};
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&per_sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&threads_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&blocks_sm, cudaDevAttrMaxBlocksPerMultiprocessor, dev) != cudaSuccess ||
      cudaFuncGetAttributes(&fa, fn) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (block < 1 || block > fa.maxThreadsPerBlock || tmem_cols < 1 || tmem_cols > 512) return 0;
  const int warps = (block + 31) / 32;
  const int regs_warp = ((((fa.numRegs > 0 ? fa.numRegs : 1) + 7) / 8 * 8) * 32 + 255) / 256 * 256;
  int v = regs_sm / (regs_warp * warps);
  v = std::min(v, threads_sm / (warps * 32));
  v = std::min(v, blocks_sm);
  const size_t per_block = (smem + fa.sharedSizeBytes + (size_t)reserved + 127) / 128 * 128;
  v = std::min(v, (int)((size_t)per_sm_smem / per_block));
  v = std::min(v, 512 / tmem_cols);
  return v < 0 ? 0 : v;
}

int grid_for(long long n, int block, int blocks_per_sm) {
  const int nsm = sm_count();
  long long need = (n + block - 1) / block;
  long long cap = (long long)nsm * blocks_per_sm;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

int pointer_access(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    a.type = cudaMemoryTypeUnregistered;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return XT_PTR_DEVICE;
  if (a.type == cudaMemoryTypeHost) return XT_PTR_PINNED;
  static int pageable = -1;
  if (pageable < 0) {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    pageable = (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess && v) ? 1 : 0;
  }
  return pageable ? XT_PTR_PAGEABLE : XT_PTR_INACCESSIBLE;
}

// ------------------------------------------------------------------ handle
struct SphHandle {
  int lmax, nmax, numr, cmap;
  double rmin, rmax, scale;
  // FP64 arrays
  double *xi = nullptr, *p0 = nullptr, *d0 = nullptr, *fact = nullptr, *rnode = nullptr;
  double *efp = nullptr, *efd = nullptr;   // [(L+1)][K][numr]
  float2* efp_df = nullptr;                 // efp split into FP32 leading part and remainder
  // FP32 copies for the mixed path
  float *xi_f = nullptr, *p0_f = nullptr, *d0_f = nullptr, *fact_f = nullptr, *rnode_f = nullptr;
  SphTab<double> tab_d;
  SphTab<float> tab_f;
};

static void free_handle(SphHandle* h) {
  if (!h) return;
  void* ptrs[] = {h->xi, h->p0, h->d0, h->fact, h->efp, h->efd, h->xi_f, h->p0_f, h->d0_f, h->fact_f,
                  h->rnode, h->rnode_f, h->efp_df};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete h;
}

template <typename T>
static int upload(T** dst, const T* src, size_t count) {
  XT_CUDA(cudaMalloc((void**)dst, count * sizeof(T)));
  XT_CUDA(cudaMemcpy(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice));
  return XT_OK;
}

static std::vector<float> to_f32(const double* a, size_t n) {
  std::vector<float> v(n);
  for (size_t i = 0; i < n; ++i) v[i] = (float)a[i];
  return v;
}

// ------------------------------------------------------------------ kernels
// expcoef[row, n] = sum_i efp[l, n, i] * D[row, i]; one block per (row, n).
__global__ void __launch_bounds__(256) k_sph_contract(const double* __restrict__ efp, const double* __restrict__ D,
                                                      int lmax, int nmax, int numr, double* __restrict__ out) {
  const int row = blockIdx.x / nmax;
  const int n = blockIdx.x % nmax;
  int l = 0;
  while ((l + 1) * (l + 1) <= row) ++l;
  const double* e = efp + ((size_t)l * nmax + n) * numr;
  const double* d = D + (size_t)row * numr;
  double acc = 0.0;
  for (int i = threadIdx.x; i < numr; i += blockDim.x) acc += e[i] * d[i];
  __shared__ double sh[32];
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if (threadIdx.x == 0) out[(size_t)row * nmax + n] = acc;
  }
}

// FP64 field (drop-in path): GH[(node*nrow + row)*2 + {0,1}] =
// sum_{n<nuse} s*c[row,n]*{efp,efd}[l,n,node] for rows with l <= luse (others 0).
__global__ void __launch_bounds__(256) k_sph_field(const double* __restrict__ efp, const double* __restrict__ efd,
                                                   const double* __restrict__ coef, double scale, int lmax, int nmax,
                                                   int numr, int luse, int nuse, double* __restrict__ GH) {
  const int nrow = (lmax + 1) * (lmax + 1);
  const long long total = (long long)numr * nrow;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int node = (int)(t / nrow);
    const int row = (int)(t % nrow);
    int l = 0;
    while ((l + 1) * (l + 1) <= row) ++l;
    double g = 0.0, h = 0.0;
    if (l <= luse) {
      for (int n = 0; n < nuse; ++n) {
        const double c = scale * coef[(size_t)row * nmax + n];
        const size_t ix = ((size_t)l * nmax + n) * numr + node;
        g += c * efp[ix];
        h += c * efd[ix];
      }
    }
    GH[2 * t] = g;
    GH[2 * t + 1] = h;
  }
}

__device__ __forceinline__ double sph_field_sum(const double* __restrict__ tab, const double* __restrict__ coef,
                                                double scale, int l, int row, int nmax, int numr, int nuse, int node) {
  double g = 0.0;
  for (int n = 0; n < nuse; ++n) g += scale * coef[(size_t)row * nmax + n] * tab[((size_t)l * nmax + n) * numr + node];
  return g;
}

// FP32 field (mixed path), SphFieldLayout<float>: per lerp base node i and
// row, float4 (G[i], G[i+1], D1[j], D2[j]), j = max(i, 1), and float2
// (Gd[i], Gd[i+1]); every entry is formed in FP64 and rounded once.  Node
// numr-1 is never a lerp base and stays zero.
__global__ void __launch_bounds__(256) k_sph_field32(const double* __restrict__ efp, const double* __restrict__ efd,
                                                     const double* __restrict__ p0, const double* __restrict__ coef,
                                                     double scale, int lmax, int nmax, int numr, int luse, int nuse,
                                                     float4* __restrict__ GA, float2* __restrict__ GD) {
  const int nrow = (lmax + 1) * (lmax + 1);
  const long long total = (long long)numr * nrow;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t / nrow);
    const int row = (int)(t % nrow);
    int l = 0;
    while ((l + 1) * (l + 1) <= row) ++l;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
    float2 d = make_float2(0.f, 0.f);
    if (l <= luse && i < numr - 1) {
      const int j = i < 1 ? 1 : i;
      const double gm = sph_field_sum(efp, coef, scale, l, row, nmax, numr, nuse, j - 1);
      const double gc = sph_field_sum(efp, coef, scale, l, row, nmax, numr, nuse, j);
      const double gp = (j + 1 < numr) ? sph_field_sum(efp, coef, scale, l, row, nmax, numr, nuse, j + 1) : 0.0;
      const double gi = (i == j) ? gc : gm, gi1 = (i == j) ? gp : gc;
      const double hm = p0[j - 1] * gm, hc = p0[j] * gc, hp = (j + 1 < numr) ? p0[j + 1] * gp : 0.0;
      a = make_float4((float)gi, (float)gi1, (float)(0.5 * (hp - hm)), (float)(hm - 2.0 * hc + hp));
      d = make_float2((float)sph_field_sum(efd, coef, scale, l, row, nmax, numr, nuse, i),
                      (float)sph_field_sum(efd, coef, scale, l, row, nmax, numr, nuse, i + 1));
    }
    GA[t] = a;
    GD[t] = d;
  }
}

bool sph_efp_df(void* handle, const float2** efp_df) {
  SphHandle* h = static_cast<SphHandle*>(handle);
  if (!h) return false;
  *efp_df = h->efp_df;
  return true;
}

bool sph_efp(void* handle, const double** efp) {
  SphHandle* h = static_cast<SphHandle*>(handle);
  if (!h) return false;
  *efp = h->efp;
  return true;
}

bool sph_tabs(void* handle, SphTab<double>* d, SphTab<float>* f) {
  SphHandle* h = static_cast<SphHandle*>(handle);
  if (!h) return false;
  if (d) *d = h->tab_d;
  if (f) *f = h->tab_f;
  return true;
}


// ------------------------------------------------------------------ allocation-free accumulation
// Some callers cannot allocate device memory for a workspace: a host
// application or framework that owns every byte of device memory through its
// own pool and forbids outside cudaMalloc, a latency-critical loop that cannot
// afford the synchronisation cudaMalloc/cudaFree may cause, or a plain C /
// cgo / Fortran binding with no device allocator to hand.  For them
// xt_sph_accumulate_noalloc keeps the deposit grid in this fixed array, which
// every GPU that loads the library holds until the process exits.
#define XT_SPH_NOALLOC_MAX_DOUBLES 262144  // 2 MiB: (lmax+1)^2 * numr must not exceed this
static __device__ __align__(256) double g_sph_noalloc_grid[XT_SPH_NOALLOC_MAX_DOUBLES];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_addr[256] = {};             // device address of the array, per device ordinal
unsigned long long g_noalloc_ctx[256] = {};   // the context it was looked up in (cuCtxGetId)

// Identifier of the calling thread's current context (unique for the
// process's lifetime), through the driver entry points the runtime exposes,
// so the library needs no link to the driver library.  False when there is
// no current context yet or the entry points are unavailable.
bool current_context_id(unsigned long long* id) {
  typedef CUresult (*GetCurrent)(CUcontext*);
  typedef CUresult (*GetId)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  });
  if (!get_current || !get_id) return false;
  CUcontext c = nullptr;
  if (get_current(&c) != CUDA_SUCCESS || !c) return false;
  return get_id(c, id) == CUDA_SUCCESS;
}
}  // namespace

// Device address of the static grid on the current device: looked up
// (cudaGetSymbolAddress with that device current) on the first call and
// again whenever the device's context has changed since, as after
// cudaDeviceReset, when the module and its array are loaded anew.
static int noalloc_grid(double** out) {
  int dev = 0;
  XT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 256) {
    set_error("device ordinal %d out of range for the static accumulation grid", dev);
    return XT_ERR_ARG;
  }
  unsigned long long id = 0;
  const bool have = current_context_id(&id);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev] || !have || g_noalloc_ctx[dev] != id) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_sph_noalloc_grid);   // creates the context if there is none
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_sph_noalloc_grid)");
    g_noalloc_addr[dev] = static_cast<double*>(p);
    g_noalloc_ctx[dev] = current_context_id(&id) ? id : 0;
  }
  *out = g_noalloc_addr[dev];
  return XT_OK;
}

}  // namespace xt

using namespace xt;

extern "C" {

int xt_abi_version(void) { return 1; }
const char* xt_last_error(void) { return xt::g_err.c_str(); }
int xt_pointer_access(const void* p) { return xt::pointer_access(p); }

int xt_copy_async(int ncopy, void* const* dst, const void* const* src, const size_t* bytes, void* stream) {
  XT_REQUIRE(ncopy >= 0 && (ncopy == 0 || (dst && src && bytes)), "NULL copy list");
  for (int i = 0; i < ncopy; ++i) {
    if (!bytes[i]) continue;
    XT_REQUIRE(dst[i] && src[i], "copy %d: NULL pointer", i);
    XT_CUDA(cudaMemcpyAsync(dst[i], src[i], bytes[i], cudaMemcpyDefault, xt::as_stream(stream)));
  }
  return XT_OK;
}

int xt_stream_sync(void* stream) {
  XT_CUDA(cudaStreamSynchronize(xt::as_stream(stream)));
  return XT_OK;
}

int xt_sph_table_create(int lmax, int nmax, int numr, int cmap, double rmin, double rmax, double scale,
                        const double* xi, const double* p0, const double* d0, const double* ev, const double* ef,
                        void** handle) {
  XT_REQUIRE(handle, "handle out-pointer is NULL");
  *handle = nullptr;
  XT_REQUIRE(lmax >= 0 && lmax <= 8, "lmax must be in [0, 8], got %d", lmax);
  XT_REQUIRE(nmax >= 1 && numr >= 3, "need nmax >= 1 and numr >= 3 (got %d, %d)", nmax, numr);
  XT_REQUIRE(cmap >= 0 && cmap <= 2, "cmap must be 0, 1 or 2");
  XT_REQUIRE(xi && p0 && d0 && ev && ef, "NULL table array");
  XT_REQUIRE(xi[1] != xi[0], "degenerate xi grid");
  SphHandle* h = new SphHandle();
  h->lmax = lmax; h->nmax = nmax; h->numr = numr; h->cmap = cmap;
  h->rmin = rmin; h->rmax = rmax; h->scale = scale;
  const size_t L1 = lmax + 1;
  std::vector<double> efp(L1 * nmax * numr), efd(L1 * nmax * numr);
  for (size_t l = 0; l < L1; ++l)
    for (int n = 0; n < nmax; ++n) {
      const double sev = sqrt(ev[l * nmax + n]);
      for (int i = 0; i < numr; ++i) {
        const size_t k = (l * nmax + n) * numr + i;
        efp[k] = ef[k] / sev;
        efd[k] = ef[k] * sev;
      }
    }
  // factorial_return (spheresl.py:823-863)
  std::vector<double> fact(L1 * L1, 0.0);
  for (int l = 0; l <= lmax; ++l)
    for (int m = 0; m <= l; ++m) {
      double f = sqrt((0.5 * l + 0.25) / PI * exp(lgamma(1.0 + l - m) - lgamma(1.0 + l + m)));
      if (m != 0) f *= sqrt(2.0);
      fact[l * L1 + m] = f;
    }
  double xi0 = xi[0];
  for (int i = 1; i < numr; ++i) xi0 = xi[i] < xi0 ? xi[i] : xi0;
  int rc;
  if ((rc = upload(&h->xi, xi, numr)) || (rc = upload(&h->p0, p0, numr)) || (rc = upload(&h->d0, d0, numr)) ||
      (rc = upload(&h->fact, fact.data(), fact.size())) || (rc = upload(&h->efp, efp.data(), efp.size())) ||
      (rc = upload(&h->efd, efd.data(), efd.size()))) {
    free_handle(h);
    return rc;
  }
  // the same table as FP32 pairs (hi, lo = rounding of the remainder) for the
  // double-float batched contraction
  {
    std::vector<float2> e2(efp.size());
    for (size_t k = 0; k < efp.size(); ++k) {
      const float hi = (float)efp[k];
      e2[k] = make_float2(hi, (float)(efp[k] - (double)hi));
    }
    if ((rc = upload(&h->efp_df, e2.data(), e2.size()))) {
      free_handle(h);
      return rc;
    }
  }
  // node radii xi_to_r(xi) (compatibility.py:54-62)
  std::vector<double> rn(numr);
  for (int i = 0; i < numr; ++i)
    rn[i] = (cmap == 1) ? (1.0 + xi[i]) / (1.0 - xi[i]) * scale : (cmap == 2 ? exp(xi[i]) : xi[i]);
  if ((rc = upload(&h->rnode, rn.data(), numr))) {
    free_handle(h);
    return rc;
  }
  auto rnf = to_f32(rn.data(), numr);
  if ((rc = upload(&h->rnode_f, rnf.data(), numr))) {
    free_handle(h);
    return rc;
  }
  auto xf = to_f32(xi, numr), pf = to_f32(p0, numr), df = to_f32(d0, numr), ff = to_f32(fact.data(), fact.size());
  if ((rc = upload(&h->xi_f, xf.data(), numr)) || (rc = upload(&h->p0_f, pf.data(), numr)) ||
      (rc = upload(&h->d0_f, df.data(), numr)) || (rc = upload(&h->fact_f, ff.data(), ff.size()))) {
    free_handle(h);
    return rc;
  }
  const double lo = (cmap == 2) ? log(rmin) : 0.0, hi = (cmap == 2) ? log(rmax) : 0.0;
  const double dxi = xi[1] - xi[0];
  h->tab_d = SphTab<double>{lmax, nmax, numr, cmap, scale, xi0, dxi, lo, hi, 1.0 / scale, 1.0 / dxi,
                            h->xi, h->p0, h->d0, h->fact, h->rnode};
  h->tab_f = SphTab<float>{lmax, nmax, numr, cmap, (float)scale, (float)xi0, (float)dxi, (float)lo, (float)hi,
                           (float)(1.0 / scale), (float)(1.0 / dxi), h->xi_f, h->p0_f, h->d0_f, h->fact_f,
                           h->rnode_f};
  *handle = h;
  return XT_OK;
}

int xt_sph_table_destroy(void* handle) {
  free_handle(static_cast<SphHandle*>(handle));
  return XT_OK;
}

size_t xt_sph_accumulate_workspace(void* handle) {
  SphHandle* h = static_cast<SphHandle*>(handle);
  if (!h) return 0;
  return (size_t)sph_nrow(h->lmax) * h->numr * sizeof(double);
}

int xt_sph_accumulate(void* handle, const double* x, const double* y, const double* z, const double* m, long long n,
                      int no_odd, int precision, double* expcoef_out, void* workspace, size_t workspace_bytes,
                      void* stream) {
  SphHandle* h = static_cast<SphHandle*>(handle);
  XT_REQUIRE(h, "NULL table handle");
  XT_REQUIRE(n >= 0, "negative particle count");
  XT_REQUIRE(expcoef_out, "NULL output");
  XT_REQUIRE(n == 0 || (x && y && z && m), "NULL particle array");
  XT_REQUIRE(precision == XT_F64 || precision == XT_F32, "bad precision %d", precision);
  const size_t need = xt_sph_accumulate_workspace(handle);
  if (!workspace || workspace_bytes < need) {
    set_error("workspace of %zu bytes needed, %zu given", need, workspace_bytes);
    return XT_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  double* D = static_cast<double*>(workspace);
  XT_CUDA(cudaMemsetAsync(D, 0, need, st));
  if (n > 0) {
    const int block = 256;
    const int grid = grid_for(n, block, 8);
    int rc = with_lcap(h->lmax, [&](auto lc) {
      constexpr int LC = decltype(lc)::value;
      if (precision == XT_F64)
        launch_sph_deposit<double, LC>(h->tab_d, x, y, z, m, n, no_odd, D, grid, block, st);
      else
        launch_sph_deposit<float, LC>(h->tab_f, x, y, z, m, n, no_odd, D, grid, block, st);
      return XT_OK;
    });
    if (rc) return rc;
    XT_CHECK_LAUNCH("k_sph_deposit");
  }
  k_sph_contract<<<sph_nrow(h->lmax) * h->nmax, 256, 0, st>>>(h->efp, D, h->lmax, h->nmax, h->numr, expcoef_out);
  XT_CHECK_LAUNCH("k_sph_contract");
  return XT_OK;
}

int xt_sph_accumulate_noalloc(void* handle, const double* x, const double* y, const double* z, const double* m,
                              long long n, int no_odd, int precision, double* expcoef_out, void* stream) {
  SphHandle* h = static_cast<SphHandle*>(handle);
  XT_REQUIRE(h, "NULL table handle");
  XT_REQUIRE(n >= 0, "negative particle count");
  XT_REQUIRE(expcoef_out, "NULL output");
  XT_REQUIRE(n == 0 || (x && y && z && m), "NULL particle array");
  XT_REQUIRE(precision == XT_F64 || precision == XT_F32, "bad precision %d", precision);
  const size_t need = (size_t)sph_nrow(h->lmax) * h->numr;
  XT_REQUIRE(need <= XT_SPH_NOALLOC_MAX_DOUBLES,
             "xt_sph_accumulate_noalloc: (lmax+1)^2 * numr = %zu exceeds the static grid of %d doubles (2 MiB); "
             "use xt_sph_accumulate with a caller workspace", need, XT_SPH_NOALLOC_MAX_DOUBLES);
  double* D = nullptr;
  int rc = noalloc_grid(&D);
  if (rc) return rc;
  cudaStream_t st = as_stream(stream);
  // the grid keeps the previous call's sums: zero the part this call uses
  XT_CUDA(cudaMemsetAsync(D, 0, need * sizeof(double), st));
  if (n > 0) {
    const int block = 256;
    const int grid = grid_for(n, block, 8);
    rc = with_lcap(h->lmax, [&](auto lc) {
      constexpr int LC = decltype(lc)::value;
      if (precision == XT_F64)
        launch_sph_deposit<double, LC>(h->tab_d, x, y, z, m, n, no_odd, D, grid, block, st);
      else
        launch_sph_deposit<float, LC>(h->tab_f, x, y, z, m, n, no_odd, D, grid, block, st);
      return XT_OK;
    });
    if (rc) return rc;
    XT_CHECK_LAUNCH("k_sph_deposit (noalloc)");
  }
  k_sph_contract<<<sph_nrow(h->lmax) * h->nmax, 256, 0, st>>>(h->efp, D, h->lmax, h->nmax, h->numr, expcoef_out);
  XT_CHECK_LAUNCH("k_sph_contract (noalloc)");
  return XT_OK;
}

size_t xt_sph_field_bytes(void* handle, int precision) {
  SphHandle* h = static_cast<SphHandle*>(handle);
  if (!h) return 0;
  return (size_t)h->numr * sph_nrow(h->lmax) *
         (precision == XT_F32 ? SphFieldLayout<float>::per_row * sizeof(float)
                              : SphFieldLayout<double>::per_row * sizeof(double));
}

int xt_sph_prepare(void* handle, const double* expcoef, double coef_scale, int lmax_use, int nmax_use, int precision,
                   void* field, size_t field_bytes, void* stream) {
  SphHandle* h = static_cast<SphHandle*>(handle);
  XT_REQUIRE(h && expcoef && field, "NULL handle, coefficients or field");
  XT_REQUIRE(precision == XT_F64 || precision == XT_F32, "bad precision %d", precision);
  if (lmax_use < 0 || lmax_use > h->lmax) lmax_use = h->lmax;
  if (nmax_use < 0 || nmax_use > h->nmax) nmax_use = h->nmax;
  const size_t need = xt_sph_field_bytes(handle, precision);
  if (field_bytes < need) {
    set_error("field buffer of %zu bytes needed, %zu given", need, field_bytes);
    return XT_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  const long long total = (long long)h->numr * sph_nrow(h->lmax);
  const int grid = grid_for(total, 256, 4);
  if (precision == XT_F64) {
    k_sph_field<<<grid, 256, 0, st>>>(h->efp, h->efd, expcoef, coef_scale, h->lmax, h->nmax, h->numr, lmax_use,
                                      nmax_use, static_cast<double*>(field));
  } else {
    float* f = static_cast<float*>(field);
    k_sph_field32<<<grid, 256, 0, st>>>(h->efp, h->efd, h->p0, expcoef, coef_scale, h->lmax, h->nmax, h->numr,
                                        lmax_use, nmax_use, reinterpret_cast<float4*>(f),
                                        reinterpret_cast<float2*>(f + (size_t)total * 4));
  }
  XT_CHECK_LAUNCH("k_sph_field");
  return XT_OK;
}

int xt_sph_eval_points(void* handle, const void* field, int precision, int coord_mode, const double* a,
                       const double* b, const double* c, long long n, int mode, int L1, int L2, int no_odd,
                       int lmax_use, int trig_l, double* const* outs, void* stream) {
  SphHandle* h = static_cast<SphHandle*>(handle);
  XT_REQUIRE(h && field && outs, "NULL handle, field or output list");
  XT_REQUIRE(n >= 0, "negative point count");
  XT_REQUIRE(n == 0 || (a && b && c), "NULL coordinate array");
  XT_REQUIRE(mode >= 0 && mode <= 2, "bad spherical eval mode %d", mode);
  XT_REQUIRE(coord_mode == XT_COORD_CART || coord_mode == XT_COORD_SPH, "bad coordinate mode");
  XT_REQUIRE(precision == XT_F64 || precision == XT_F32, "bad precision %d", precision);
  if (n == 0) return XT_OK;
  if (lmax_use < 0 || lmax_use > h->lmax) lmax_use = h->lmax;
  SphEvalOpts o;
  o.mode = mode; o.L1 = L1; o.L2 = L2; o.no_odd = no_odd; o.lmax_use = lmax_use; o.trig_l = trig_l;
  o.want_dens = (mode != XT_SPH_FORCE_EVAL) && (outs[0] || outs[1]);
  cudaStream_t st = as_stream(stream);
  const int block = 128;
  const int grid = grid_for(n, block, 8);
  int rc = with_lcap(h->lmax, [&](auto lc) {
    constexpr int LC = decltype(lc)::value;
    if (precision == XT_F64)
      launch_sph_eval<double, LC>(h->tab_d, static_cast<const double*>(field), coord_mode, a, b, c, n, o, outs, grid,
                                  block, st);
    else
      launch_sph_eval<float, LC>(h->tab_f, static_cast<const float*>(field), coord_mode, a, b, c, n, o, outs, grid,
                                 block, st);
    return XT_OK;
  });
  if (rc) return rc;
  XT_CHECK_LAUNCH("k_sph_eval");
  return XT_OK;
}

}  // extern "C"
