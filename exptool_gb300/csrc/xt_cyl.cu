// Cylindrical EOF basis: table upload, coefficient accumulation, evaluation.
//
// Accumulation (eof.accumulate, eof.py:492-640) is reorganised as a bilinear
// deposition: each particle adds -4 pi m {cos, sin}(m phi) times its four
// bilinear weights to a node grid D[m][cs][node]; one memory-bound pass then
// contracts the grid with the potential tables,
//     cos[m, n] = sum_node potC[m, n, node] * D[m][0][node]
//     sin[m, n] = sum_node potS[m, n, node] * D[m][1][node],
// which is the reference sum (eof.py:534-551) with the bilinear interpolation
// (linear in the table values) moved after the particle sum.  Evaluation
// contracts the coefficients with the tables into per-node fields first
// (cos/sin-weighted pot, rforce, zforce[, dens] per m), so each particle
// reads 4 corners x (mmax+1) x 6 values instead of 4 x 6 x (mmax+1) x norder.
#include <cstring>
#include <type_traits>
#include <vector>

#include "xt_internal.cuh"

namespace xt {

struct CylHandle {
  int mmax, norder, numx, numy, cmap, dens;
  double XMIN, dX, YMIN, dY, ascale, hscale;
  size_t nnode;
  double* tab = nullptr;   // [8][mmax+1][norder][nnode]: potC rforceC zforceC densC potS rforceS zforceS densS
  CylTab<double> tab_d;
  CylTab<float> tab_f;
};

static inline const double* tab_ptr(const CylHandle* h, int which) {
  return h->tab + (size_t)which * (h->mmax + 1) * h->norder * h->nnode;
}

constexpr double FOUR_PI_C = 4.0 * PI;

// One thread per particle; FP64 atomics onto D[(m*2 + cs)*nnode + node].
template <typename R>
__global__ void __launch_bounds__(256) k_cyl_deposit(CylTab<R> T, const double* __restrict__ x,
                                                     const double* __restrict__ y, const double* __restrict__ z,
                                                     const double* __restrict__ mass, long long n,
                                                     double* __restrict__ D, size_t nnode) {
  const int ny1 = T.numy + 1;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const R xx = (R)x[p], yy = (R)y[p], zz = (R)z[p];
    const R Rc = sqrt(xx * xx + yy * yy + R(1.0e-10));
    R c1, s1;
    unit_phi(xx, yy, c1, s1);
    const CylBins<R> B = cyl_bins(T, Rc, zz);
    const R base = R(-FOUR_PI_C) * (R)mass[p];
    const size_t n00 = B.node, n10 = n00 + ny1, n01 = n00 + 1, n11 = n10 + 1;
    R cprev = R(1), sprev = R(0), ccur = c1, scur = s1;
    for (int m = 0; m <= T.mmax; ++m) {
      R c, s;
      if (m == 0) { c = R(1); s = R(0); }
      else if (m == 1) { c = c1; s = s1; }
      else {
        c = R(2) * c1 * ccur - cprev;
        s = R(2) * c1 * scur - sprev;
        cprev = ccur; sprev = scur; ccur = c; scur = s;
      }
      const R wc = base * c;
      double* dc = D + (size_t)(2 * m) * nnode;
      atomicAdd(dc + n00, (double)(wc * B.c00));
      atomicAdd(dc + n10, (double)(wc * B.c10));
      atomicAdd(dc + n01, (double)(wc * B.c01));
      atomicAdd(dc + n11, (double)(wc * B.c11));
      if (m > 0) {
        const R ws = base * s;
        double* ds = dc + nnode;
        atomicAdd(ds + n00, (double)(ws * B.c00));
        atomicAdd(ds + n10, (double)(ws * B.c10));
        atomicAdd(ds + n01, (double)(ws * B.c01));
        atomicAdd(ds + n11, (double)(ws * B.c11));
      }
    }
  }
}

// Partial dot products: block (chunk, out) with out = (m*norder + k)*2 + cs.
__global__ void __launch_bounds__(256) k_cyl_contract_partial(const double* __restrict__ potC,
                                                              const double* __restrict__ potS,
                                                              const double* __restrict__ D, int mmax, int norder,
                                                              size_t nnode, int nchunk, double* __restrict__ part) {
  const int chunk = blockIdx.x;
  const int out = blockIdx.y;
  const int cs = out & 1;
  const int mk = out >> 1;
  const int m = mk / norder;
  double acc = 0.0;
  if (!(cs == 1 && m == 0)) {
    const double* t = (cs ? potS : potC) + (size_t)mk * nnode;
    const double* d = D + (size_t)(2 * m + cs) * nnode;
    const size_t per = (nnode + nchunk - 1) / nchunk;
    const size_t lo = (size_t)chunk * per;
    const size_t hi = lo + per < nnode ? lo + per : nnode;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) acc += t[i] * d[i];
  }
  __shared__ double sh[32];
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if (threadIdx.x == 0) part[(size_t)out * nchunk + chunk] = acc;
  }
}

// Fixed-order sum of the partials: cos[m,k], sin[m,k].
__global__ void k_cyl_contract_final(const double* __restrict__ part, int nout, int nchunk, double* __restrict__ cos_out,
                                     double* __restrict__ sin_out) {
  const int out = blockIdx.x * blockDim.x + threadIdx.x;
  if (out >= nout) return;
  double acc = 0.0;
  for (int c = 0; c < nchunk; ++c) acc += part[(size_t)out * nchunk + c];
  const int mk = out >> 1;
  if (out & 1) sin_out[mk] = acc;
  else cos_out[mk] = acc;
}

// Fields F[(node*(mmax+1) + m)*nf + f] for m <= muse (m > muse left 0).
// A block owns TN consecutive nodes; thread t reads table rows coalesced
// along nodes and the tile is written back contiguously through shared memory.
template <typename R, int TN>
__global__ void __launch_bounds__(256) k_cyl_field(const double* __restrict__ tab, const double* __restrict__ cosc,
                                                   const double* __restrict__ sinc, int mmax, int norder,
                                                   size_t nnode, int muse, int nuse, int nf, R* __restrict__ F) {
  extern __shared__ unsigned char smem_raw[];
  R* tile = reinterpret_cast<R*>(smem_raw);
  const int mf_total = (mmax + 1) * nf;
  const size_t node0 = (size_t)blockIdx.x * TN;
  const size_t tsize = (size_t)(mmax + 1) * norder * nnode;
  // table index of field f: PC RC ZC PS RS ZS DC DS -> 0 1 2 4 5 6 3 7
  const int tmap[8] = {0, 1, 2, 4, 5, 6, 3, 7};
  for (int idx = threadIdx.x; idx < TN * mf_total; idx += blockDim.x) {
    const int nl = idx % TN;
    const int mf = idx / TN;
    const int m = mf / nf, f = mf % nf;
    const size_t node = node0 + nl;
    double acc = 0.0;
    if (node < nnode && m <= muse && !(m == 0 && (f == 3 || f == 4 || f == 5 || f == 7))) {
      const int ti = tmap[f];
      const double* coef = (ti >= 4) ? sinc : cosc;
      const double* t = tab + (size_t)ti * tsize + (size_t)m * norder * nnode + node;
      for (int k = 0; k < nuse; ++k) acc += coef[m * norder + k] * t[(size_t)k * nnode];
    }
    tile[nl * mf_total + mf] = (R)acc;
  }
  __syncthreads();
  const size_t nvalid = (node0 + TN <= nnode) ? TN : (nnode - node0);
  R* dst = F + node0 * mf_total;
  for (int idx = threadIdx.x; idx < (int)(nvalid * mf_total); idx += blockDim.x) dst[idx] = tile[idx];
}

template <typename R>
__global__ void __launch_bounds__(128) k_cyl_eval(CylTab<R> T, const R* __restrict__ F, int coord_mode,
                                                  const double* __restrict__ a, const double* __restrict__ b,
                                                  const double* __restrict__ c, long long n, CylEvalOpts o,
                                                  double* o0, double* o1, double* o2, double* o3, double* o4,
                                                  double* o5, double* o6, double* o7) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    R Rc, zz, c1, s1;
    if (coord_mode == XT_COORD_CART) {
      const R xx = (R)a[p], yy = (R)b[p];
      zz = (R)c[p];
      Rc = sqrt(xx * xx + yy * yy + R(1.0e-10));
      unit_phi(xx, yy, c1, s1);
    } else {
      Rc = (R)a[p];
      zz = (R)b[p];
      sincos_r((R)c[p], &s1, &c1);
    }
    R v[9];
    cyl_eval_point<R, 16>(T, F, Rc, zz, c1, s1, o, v);
    // v = p0 p fr fp fz d0 d fr0 fz0
    if (o.mode == XT_CYL_ACCUMULATED_EVAL_PARTICLES) {
      if (o0) o0[p] = v[0];
      if (o1) o1[p] = v[1];
      if (o2) o2[p] = v[2];
      if (o3) o3[p] = v[3];
      if (o4) o4[p] = v[4];
      if (o5) o5[p] = (double)Rc;
      if (o6) o6[p] = v[5];
      if (o7) o7[p] = v[6];
    } else if (o.mode == XT_CYL_FORCE_EVAL) {
      if (o.perturb) {  // fr fp fz p p0 fr0 fz0
        if (o0) o0[p] = v[2];
        if (o1) o1[p] = v[3];
        if (o2) o2[p] = v[4];
        if (o3) o3[p] = v[1];
        if (o4) o4[p] = v[0];
        if (o5) o5[p] = v[7];
        if (o6) o6[p] = v[8];
      } else {          // fr+fr0 fp fz+fz0 p+p0 p0
        if (o0) o0[p] = (double)(v[2] + v[7]);
        if (o1) o1[p] = v[3];
        if (o2) o2[p] = (double)(v[4] + v[8]);
        if (o3) o3[p] = (double)(v[1] + v[0]);
        if (o4) o4[p] = v[0];
      }
    } else {  // ACCUMULATED_EVAL: p0 p fr fp fz d0 d
      if (o0) o0[p] = v[0];
      if (o1) o1[p] = v[1];
      if (o2) o2[p] = v[2];
      if (o3) o3[p] = v[3];
      if (o4) o4[p] = v[4];
      if (o5) o5[p] = v[5];
      if (o6) o6[p] = v[6];
    }
  }
}

static const int kContractChunks = 8;

bool cyl_tabs(void* handle, CylTab<double>* d, CylTab<float>* f) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  if (!h) return false;
  if (d) *d = h->tab_d;
  if (f) *f = h->tab_f;
  return true;
}

}  // namespace xt

using namespace xt;

extern "C" {

int xt_cyl_table_create(int mmax, int norder, int numx, int numy, int cmap, int dens, double XMIN, double dX,
                        double YMIN, double dY, double ascale, double hscale, const double* potC,
                        const double* rforceC, const double* zforceC, const double* densC, const double* potS,
                        const double* rforceS, const double* zforceS, const double* densS, void** handle) {
  XT_REQUIRE(handle, "handle out-pointer is NULL");
  *handle = nullptr;
  XT_REQUIRE(mmax >= 0 && mmax <= 64 && norder >= 1, "bad mmax %d / norder %d", mmax, norder);
  XT_REQUIRE(numx >= 1 && numy >= 1, "numx, numy must be >= 1");
  XT_REQUIRE(cmap >= 0 && cmap <= 2, "cmap must be 0, 1 or 2");
  XT_REQUIRE(dX != 0.0 && dY != 0.0, "degenerate table spacing");
  XT_REQUIRE(potC && potS, "NULL potential table");
  XT_REQUIRE(!dens || (densC && densS), "density tables required when dens != 0");
  CylHandle* h = new CylHandle();
  h->mmax = mmax; h->norder = norder; h->numx = numx; h->numy = numy; h->cmap = cmap; h->dens = dens ? 1 : 0;
  h->XMIN = XMIN; h->dX = dX; h->YMIN = YMIN; h->dY = dY; h->ascale = ascale; h->hscale = hscale;
  h->nnode = (size_t)(numx + 1) * (numy + 1);
  const size_t tsize = (size_t)(mmax + 1) * norder * h->nnode;
  cudaError_t e = cudaMalloc((void**)&h->tab, 8 * tsize * sizeof(double));
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(e, "cudaMalloc(EOF tables)");
  }
  // force tables may be NULL (accumulation-only handles): stored as zeros
  const double* src[8] = {potC, rforceC, zforceC, dens ? densC : nullptr, potS, rforceS, zforceS,
                          dens ? densS : nullptr};
  for (int k = 0; k < 8; ++k) {
    if (src[k]) e = cudaMemcpy(h->tab + k * tsize, src[k], tsize * sizeof(double), cudaMemcpyHostToDevice);
    else e = cudaMemset(h->tab + k * tsize, 0, tsize * sizeof(double));
    if (e != cudaSuccess) {
      cudaFree(h->tab);
      delete h;
      return cuda_fail(e, "upload EOF tables");
    }
  }
  h->tab_d = CylTab<double>{mmax, norder, numx, numy, cmap, XMIN, dX, YMIN, dY, ascale, hscale};
  h->tab_f = CylTab<float>{mmax, norder, numx, numy, cmap, (float)XMIN, (float)dX, (float)YMIN, (float)dY,
                           (float)ascale, (float)hscale};
  *handle = h;
  return XT_OK;
}

int xt_cyl_table_destroy(void* handle) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  if (h) {
    if (h->tab) cudaFree(h->tab);
    delete h;
  }
  return XT_OK;
}

size_t xt_cyl_accumulate_workspace(void* handle) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  if (!h) return 0;
  const size_t grid = (size_t)(h->mmax + 1) * 2 * h->nnode;
  const size_t part = (size_t)(h->mmax + 1) * h->norder * 2 * kContractChunks;
  return (grid + part) * sizeof(double);
}

int xt_cyl_accumulate(void* handle, const double* x, const double* y, const double* z, const double* m, long long n,
                      int precision, double* cos_out, double* sin_out, void* workspace, size_t workspace_bytes,
                      void* stream) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  XT_REQUIRE(h, "NULL table handle");
  XT_REQUIRE(n >= 0, "negative particle count");
  XT_REQUIRE(cos_out && sin_out, "NULL output");
  XT_REQUIRE(n == 0 || (x && y && z && m), "NULL particle array");
  XT_REQUIRE(precision == XT_F64 || precision == XT_F32, "bad precision %d", precision);
  const size_t need = xt_cyl_accumulate_workspace(handle);
  if (!workspace || workspace_bytes < need) {
    set_error("workspace of %zu bytes needed, %zu given", need, workspace_bytes);
    return XT_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  double* D = static_cast<double*>(workspace);
  const size_t grid_elems = (size_t)(h->mmax + 1) * 2 * h->nnode;
  double* part = D + grid_elems;
  XT_CUDA(cudaMemsetAsync(D, 0, grid_elems * sizeof(double), st));
  if (n > 0) {
    const int block = 256;
    const int grid = grid_for(n, block, 8);
    if (precision == XT_F64)
      k_cyl_deposit<double><<<grid, block, 0, st>>>(h->tab_d, x, y, z, m, n, D, h->nnode);
    else
      k_cyl_deposit<float><<<grid, block, 0, st>>>(h->tab_f, x, y, z, m, n, D, h->nnode);
    XT_CHECK_LAUNCH("k_cyl_deposit");
  }
  const int nout = (h->mmax + 1) * h->norder * 2;
  dim3 g(kContractChunks, nout);
  k_cyl_contract_partial<<<g, 256, 0, st>>>(tab_ptr(h, 0), tab_ptr(h, 4), D, h->mmax, h->norder, h->nnode,
                                            kContractChunks, part);
  XT_CHECK_LAUNCH("k_cyl_contract_partial");
  k_cyl_contract_final<<<(nout + 127) / 128, 128, 0, st>>>(part, nout, kContractChunks, cos_out, sin_out);
  XT_CHECK_LAUNCH("k_cyl_contract_final");
  return XT_OK;
}

size_t xt_cyl_field_bytes(void* handle, int density, int precision) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  if (!h) return 0;
  const int nf = density ? 8 : 6;
  return h->nnode * (h->mmax + 1) * nf * (precision == XT_F32 ? sizeof(float) : sizeof(double));
}

int xt_cyl_prepare(void* handle, const double* cos_c, const double* sin_c, int mmax_use, int nmax_use, int density,
                   int precision, void* field, size_t field_bytes, void* stream) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  XT_REQUIRE(h && cos_c && sin_c && field, "NULL handle, coefficients or field");
  XT_REQUIRE(precision == XT_F64 || precision == XT_F32, "bad precision %d", precision);
  XT_REQUIRE(!density || h->dens, "density requested but the table has no density terms");
  if (mmax_use < 0 || mmax_use > h->mmax) mmax_use = h->mmax;
  if (nmax_use < 0 || nmax_use > h->norder) nmax_use = h->norder;
  const size_t need = xt_cyl_field_bytes(handle, density, precision);
  if (field_bytes < need) {
    set_error("field buffer of %zu bytes needed, %zu given", need, field_bytes);
    return XT_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  const int nf = density ? 8 : 6;
  constexpr int TN = 32;
  const int blocks = (int)((h->nnode + TN - 1) / TN);
  const size_t mf = (size_t)(h->mmax + 1) * nf;
  if (precision == XT_F64) {
    const size_t sm = TN * mf * sizeof(double);
    if (sm > 48 * 1024) XT_CUDA(cudaFuncSetAttribute(k_cyl_field<double, TN>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_cyl_field<double, TN><<<blocks, 256, sm, st>>>(h->tab, cos_c, sin_c, h->mmax, h->norder, h->nnode, mmax_use,
                                                    nmax_use, nf, static_cast<double*>(field));
  } else {
    const size_t sm = TN * mf * sizeof(float);
    if (sm > 48 * 1024) XT_CUDA(cudaFuncSetAttribute(k_cyl_field<float, TN>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_cyl_field<float, TN><<<blocks, 256, sm, st>>>(h->tab, cos_c, sin_c, h->mmax, h->norder, h->nnode, mmax_use,
                                                   nmax_use, nf, static_cast<float*>(field));
  }
  XT_CHECK_LAUNCH("k_cyl_field");
  return XT_OK;
}

int xt_cyl_eval_points(void* handle, const void* field, int precision, int density, int coord_mode, const double* a,
                       const double* b, const double* c, long long n, int mode, int m1, int m2, int mmax_use,
                       int no_odd, int perturb, double* const* outs, void* stream) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  XT_REQUIRE(h && field && outs, "NULL handle, field or output list");
  XT_REQUIRE(n >= 0, "negative point count");
  XT_REQUIRE(n == 0 || (a && b && c), "NULL coordinate array");
  XT_REQUIRE(mode >= 0 && mode <= 2, "bad cylindrical eval mode %d", mode);
  XT_REQUIRE(coord_mode == XT_COORD_CART || coord_mode == XT_COORD_CYL, "bad coordinate mode");
  XT_REQUIRE(precision == XT_F64 || precision == XT_F32, "bad precision %d", precision);
  XT_REQUIRE(!density || h->dens, "density requested but the table has no density terms");
  if (n == 0) return XT_OK;
  if (mmax_use < 0 || mmax_use > h->mmax) mmax_use = h->mmax;
  CylEvalOpts o;
  o.mode = mode; o.m1 = m1; o.m2 = m2; o.mmax_use = mmax_use; o.no_odd = no_odd; o.perturb = perturb;
  o.density = density; o.nf = density ? 8 : 6;
  cudaStream_t st = as_stream(stream);
  const int block = 128;
  const int grid = grid_for(n, block, 8);
  if (precision == XT_F64)
    k_cyl_eval<double><<<grid, block, 0, st>>>(h->tab_d, static_cast<const double*>(field), coord_mode, a, b, c, n,
                                               o, outs[0], outs[1], outs[2], outs[3], outs[4], outs[5], outs[6],
                                               outs[7]);
  else
    k_cyl_eval<float><<<grid, block, 0, st>>>(h->tab_f, static_cast<const float*>(field), coord_mode, a, b, c, n, o,
                                              outs[0], outs[1], outs[2], outs[3], outs[4], outs[5], outs[6],
                                              outs[7]);
  XT_CHECK_LAUNCH("k_cyl_eval");
  return XT_OK;
}

}  // extern "C"
