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
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cmath>
#include <mutex>
#include <cstring>
#include <type_traits>
#include <vector>

#include "xt_df.cuh"
#include "xt_internal.cuh"
#include "xt_tc.cuh"

namespace xt {

// CUDA graph of one fused accumulate + evaluate call (xt_cyl_accumulate_eval),
// replayed while everything but the particle arrays and R stays the same;
// those five pointers are patched into the captured binning node.
struct FusedGraph {
  struct Key {
    long long n;
    int precision, m1, m2, nan_to_origin;
    const void* ws;
    const double *cos_out, *sin_out;
    double* outs[5];   // compared only for device results (qchunk = 0): staged results are copied outside
    int field_engine;
    int qchunk;
    bool same(const Key& o) const {
      if (n != o.n || precision != o.precision || m1 != o.m1 || m2 != o.m2 || nan_to_origin != o.nan_to_origin ||
          ws != o.ws || cos_out != o.cos_out || sin_out != o.sin_out || field_engine != o.field_engine ||
          qchunk != o.qchunk)
        return false;
      if (qchunk) return true;
      for (int i = 0; i < 5; ++i)
        if (outs[i] != o.outs[i]) return false;
      return true;
    }
  };
  bool valid = false;
  Key key{};
  bool seen = false;                  // `last` was run directly once: capture if it repeats
  Key last{};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t binrec = nullptr;   // the binning kernel's node in `graph`
  cudaKernelNodeParams bp{};          // its launch shape as captured
  const double *x = nullptr, *y = nullptr, *z = nullptr, *m = nullptr;
  double* rout = nullptr;
  void clear() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    binrec = nullptr;
    valid = false;
  }
};

// Parts of the particle range whose results, bound for host memory, are
// evaluated and copied out in turn (measured on 1e6 disc particles: two halves
// save 0.046 ms per call against evaluating then copying, four quarters 0.032
// ms: each part adds deposit segments, scan buckets and an evaluation launch).
// The first part holds 3/8 of the particles: the copy out runs at about half
// the evaluation's rate, so a smaller first part starts it sooner, and the
// second part's evaluation (5/8) still ends before the first part's copy.
constexpr int kHostParts = 2;

struct CylHandle {
  int mmax, norder, numx, numy, cmap, dens;
  double XMIN, dX, YMIN, dY, ascale, hscale;
  size_t nnode;
  double* tab = nullptr;   // [8][mmax+1][norder][nnode]: potC rforceC zforceC densC potS rforceS zforceS densS
  float* tab_f32 = nullptr;  // the same tables rounded to FP32 (separate mixed path), rows of pitch_f nodes
  size_t pitch_f = 0;        // row pitch of tab_f32 and of the deposit grids: nnode rounded up to 4
  // Tables of the fused paths, tiled by blocks of kTileNodes nodes: block b
  // holds, for rows r = (f * (mmax+1) + m) * norder + k with f = potC rforceC
  // zforceC potS rforceS zforceS, the entries of nodes b*kTileNodes ... as
  // FP32 roundings (tile_hi) and 16-bit remainders (tile_lo, lo16_unscaled).
  float* tile_hi = nullptr;
  short* tile_lo = nullptr;
  size_t tile_rows = 0;      // 6 (mmax+1) norder
  CylTab<double> tab_d;
  CylTab<float> tab_f;
  std::mutex graph_mu;       // guards fused and capture
  FusedGraph fused;
  cudaStream_t capture = nullptr;   // private stream the fused graph is captured on
  // Results bound for host memory are copied out part by part on `copy` while
  // the next part is evaluated (events qev: part evaluated, qdone: all copies
  // issued); copy_mu serialises the calls that use them.
  std::mutex copy_mu;
  cudaStream_t copy = nullptr;
  cudaEvent_t qev[kHostParts] = {};
  cudaEvent_t qdone = nullptr;
};

static inline const double* tab_ptr(const CylHandle* h, int which) {
  return h->tab + (size_t)which * (h->mmax + 1) * h->norder * h->nnode;
}

static inline const float* tab_ptr_f32(const CylHandle* h, int which) {
  return h->tab_f32 + (size_t)which * (h->mmax + 1) * h->norder * h->pitch_f;
}

// hi = FP32 rounding of a, rows of nnode entries re-laid with a pitch of
// `pitch` entries (padding zeroed); table set-up, once.
__global__ void k_split_tab(const double* __restrict__ a, float* __restrict__ hi, size_t rows, size_t nnode,
                            size_t pitch) {
  const size_t n = rows * pitch;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t row = i / pitch, node = i - row * pitch;
    hi[i] = node < nnode ? (float)a[row * nnode + node] : 0.f;
  }
}

constexpr int kTileNodes = 64;   // nodes per block of the tiled fused tables

// The tiled tables take the nodes in rows of constant z: tile position
// t = iy * (numx + 1) + ix holds node ix * (numy + 1) + iy, and a block is 64
// consecutive positions.  A disc fills a band of z rows, so fewer blocks
// touch its cells than with runs along z (429 against 632 of 1033 blocks for
// the 1e6-particle exponential disc on the 257^2 table).
struct TileOrder {
  int nx1, ny1;   // numx + 1, numy + 1
  __host__ __device__ size_t node(size_t t) const {
    const size_t iy = t / nx1;
    return (t - iy * nx1) * ny1 + iy;
  }
  __host__ __device__ size_t pos(int ix, int iy) const { return (size_t)iy * nx1 + ix; }
};

// Tiled fused tables (CylHandle::tile_hi/tile_lo) from the FP64 tables a
// ([8][mmax+1][norder][nnode]); entries past nnode are zero.  Set-up, once.
__global__ void k_tile_tab(const double* __restrict__ a, float* __restrict__ hi, short* __restrict__ lo,
                           int nmk, size_t nnode, size_t nblk, TileOrder to) {
  const size_t rows = 6 * (size_t)nmk;
  const size_t n = nblk * rows * kTileNodes;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t b = i / (rows * kTileNodes), rem = i - b * rows * kTileNodes;
    const size_t row = rem / kTileNodes, tp = b * kTileNodes + (rem - row * kTileNodes);
    const int f = (int)(row / nmk), mk = (int)(row - (size_t)f * nmk);
    const int t = f < 3 ? f : f + 1;                       // skip densC
    float h = 0.f;
    short l = 0;
    if (tp < nnode) {
      const double v = a[((size_t)t * nmk + mk) * nnode + to.node(tp)];
      h = (float)v;
      l = lo16_encode(v, h);
    }
    hi[i] = h;
    lo[i] = l;
  }
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
// (tables' rows are tpitch entries apart)
template <typename TT>
__global__ void __launch_bounds__(256) k_cyl_contract_partial(const TT* __restrict__ potC,
                                                              const TT* __restrict__ potS,
                                                              const double* __restrict__ D, int mmax, int norder,
                                                              size_t nnode, size_t tpitch, int nchunk,
                                                              double* __restrict__ part) {
  const int chunk = blockIdx.x;
  const int out = blockIdx.y;
  const int cs = out & 1;
  const int mk = out >> 1;
  const int m = mk / norder;
  double acc = 0.0;
  if (!(cs == 1 && m == 0)) {
    const TT* t = (cs ? potS : potC) + (size_t)mk * tpitch;
    const double* d = D + (size_t)(2 * m + cs) * nnode;
    const size_t per = (nnode + nchunk - 1) / nchunk;
    const size_t lo = (size_t)chunk * per;
    const size_t hi = lo + per < nnode ? lo + per : nnode;
    const size_t step = blockDim.x;
    size_t i = lo + threadIdx.x;
    double a1 = 0.0, a2 = 0.0, a3 = 0.0;
    for (; i + 3 * step < hi; i += 4 * step) {
      const TT t0 = t[i], t1 = t[i + step], t2 = t[i + 2 * step], t3 = t[i + 3 * step];
      const double d0 = d[i], d1 = d[i + step], d2 = d[i + 2 * step], d3 = d[i + 3 * step];
      acc += (double)t0 * d0;
      a1 += (double)t1 * d1;
      a2 += (double)t2 * d2;
      a3 += (double)t3 * d3;
    }
    for (; i < hi; i += step) acc += (double)t[i] * d[i];
    acc += a1 + a2 + a3;
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
// mzero_sin: norder when the m = 0 sine partials were not written (their
// sums are zero), else 0.
__global__ void k_cyl_contract_final(const double* __restrict__ part, int nout, int nchunk, double* __restrict__ cos_out,
                                     double* __restrict__ sin_out, int mzero_sin) {
  const int out = blockIdx.x * blockDim.x + threadIdx.x;
  if (out >= nout) return;
  if (mzero_sin && (out & 1) && (out >> 1) < mzero_sin) {   // m = 0 sine: no partials, zero
    sin_out[out >> 1] = 0.0;
    return;
  }
  double acc = 0.0;
  for (int c = 0; c < nchunk; ++c) acc += part[(size_t)out * nchunk + c];
  const int mk = out >> 1;
  if (out & 1) sin_out[mk] = acc;
  else cos_out[mk] = acc;
}

// Fields F[(node*(mmax+1) + m)*nf + f] for m <= muse (m > muse left 0).
// A block owns TN consecutive nodes; thread t reads table rows coalesced
// along nodes and the tile is written back contiguously through shared memory.
// (table rows tpitch entries apart)
template <typename R, int TN, typename TT>
__global__ void __launch_bounds__(256) k_cyl_field(const TT* __restrict__ tab, const double* __restrict__ cosc,
                                                   const double* __restrict__ sinc, int mmax, int norder,
                                                   size_t nnode, size_t tpitch, int muse, int nuse, int nf,
                                                   R* __restrict__ F) {
  extern __shared__ unsigned char smem_raw[];
  R* tile = reinterpret_cast<R*>(smem_raw);
  const int mf_total = (mmax + 1) * nf;
  const size_t node0 = (size_t)blockIdx.x * TN;
  const size_t tsize = (size_t)(mmax + 1) * norder * tpitch;
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
      const TT* t = tab + (size_t)ti * tsize + (size_t)m * norder * tpitch + node;
      int k = 0;
      for (; k + 8 <= nuse; k += 8) {     // eight table rows in flight, then the FMAs in order
        TT v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = t[(size_t)(k + u) * tpitch];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc += coef[m * norder + k + u] * (double)v[u];
      }
      for (; k < nuse; ++k) acc += coef[m * norder + k] * (double)t[(size_t)k * tpitch];
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


// ------------------------------------------------------------------ fused accumulate + evaluate
// Used when coefficients are accumulated from, and forces evaluated at, the
// same particles (eof.compute_coefficients followed by eof.compute_forces on
// one snapshot).  The per-particle set-up (maps, bins, bilinear weights,
// cos/sin phi) is computed once; particles are counting-sorted by table cell
// so that warps deposit into and gather from the same few nodes.

// One binned particle, stored whole (48 bytes as double-float, 32 as FP32) so
// that binning, sorting and both consumers move it with 16-byte accesses: the
// fractional cell coordinates dx = X - ix, dy = Y - iy (the bilinear weights
// are products of dx, dy and their complements), cos phi, sin phi, -4 pi m,
// the cell, and an index (the particle's slot within its cell as binned, its
// original index once sorted).
template <typename RT>
struct BinRec;
template <>
struct alignas(16) BinRec<df> {
  df dx, dy, c1, s1, base;
  int cell, idx;
};
template <>
struct alignas(16) BinRec<float> {
  float dx, dy, c1, s1, base;
  int cell, idx, pad;
};
static_assert(sizeof(BinRec<df>) == 48 && sizeof(BinRec<float>) == 32, "record sizes");

// Counting-sort bucket of particle p in table cell `cell`: the cell alone, or
// with qchunk > 0 (results bound for host memory) the cell within the
// particle's part min(p / qchunk, kHostParts - 1) of the particle range, so
// that the records of each part are contiguous and its results complete as a
// block.
__device__ __forceinline__ int sort_bucket(long long p, int qchunk, int ncell, int cell) {
  if (qchunk <= 0) return cell;
  int q = 0;   // p / qchunk by comparisons (below kHostParts)
#pragma unroll
  for (int j = 1; j < kHostParts; ++j) q += p >= (long long)j * qchunk ? 1 : 0;
  return q * ncell + cell;
}

template <typename R>
__device__ __forceinline__ void weights_from_frac(R dx, R dy, R w[4]) {
  const R ex = R(1) - dx, ey = R(1) - dy;
  w[0] = ex * ey;   // c00 = (ix+1-X)(iy+1-Y)
  w[1] = dx * ey;   // c10
  w[2] = ex * dy;   // c01
  w[3] = dx * dy;   // c11
}

// FP32-path record kernel (mixed precision).
template <typename R>
__global__ void __launch_bounds__(256) k_cyl_binrec(CylTab<R> T, const double* __restrict__ x,
                                                    const double* __restrict__ y, const double* __restrict__ z,
                                                    const double* __restrict__ mass, long long n,
                                                    int* __restrict__ hist, BinRec<R>* __restrict__ rec,
                                                    double* __restrict__ Rout, int nan_to_origin,
                                                    double* __restrict__ zD, float* __restrict__ zE, long long nz,
                                                    int qchunk) {
  // zero the deposit grids (read by the deposit three kernels later)
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nz; i += (long long)gridDim.x * blockDim.x) {
    zD[i] = 0.0;
    zE[i] = 0.f;
  }
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    R xx = (R)x[p], yy = (R)y[p], zz = (R)z[p];
    // eof.compute_coefficients places particles with NaN coordinates at the origin (eof.py:1189-1204)
    if (nan_to_origin && (isnan(xx) || isnan(yy) || isnan(zz))) xx = yy = zz = R(0);
    const R Rc = sqrt(xx * xx + yy * yy + R(1.0e-10));
    R c1, s1;
    unit_phi(xx, yy, c1, s1);
    // the mapping and clamps of cyl_bins (eof.return_bins), keeping X - ix and Y - iy
    R X = (r_to_xi_inv(Rc, T.cmap, T.inv_ascale) - T.XMIN) * T.inv_dX;
    R Y = (z_to_y_inv(zz, T.inv_hscale) - T.YMIN) * T.inv_dY;
    R fx = trunc(X), fy = trunc(Y);
    if (!(fx >= R(0))) fx = R(0);
    if (!(fy >= R(0))) fy = R(0);
    if (X < R(0)) X = R(0);
    if (Y < R(0)) Y = R(0);
    if (fx >= R(T.numx)) fx = R(T.numx - 1);
    if (fy >= R(T.numy)) fy = R(T.numy - 1);
    const int ix = (int)fx, iy = (int)fy;
    BinRec<R> r;
    r.dx = X - fx;
    r.dy = Y - fy;
    r.c1 = c1;
    r.s1 = s1;
    r.base = R(-FOUR_PI_C) * (R)mass[p];
    r.cell = ix * T.numy + iy;
    r.idx = atomicAdd(hist + sort_bucket(p, qchunk, T.numx * T.numy, r.cell), 1);
    rec[p] = r;
    if (Rout) Rout[p] = (double)Rc;
  }
}

// FP64-path record kernel.  The set-up of every particle (R, rho = |(x, y)|,
// cos/sin phi, the radial map including cmap = 2's log, the z map's sign
// factor and asinh, the cell and the in-cell offsets) runs in double-float
// arithmetic on the FP32 pipe: inputs are split into float pairs with
// integer operations and the returned R is assembled with one FP64 add.  Results equal the
// FP64 arithmetic to ~2^-46 relative.  Points outside the range where FP32
// exponents are safe (|x|, |y|, |z| < 1e15, rho^2 > 1e-30, coordinates 0 or
// >= 2^-74 in magnitude) take the FP64 arithmetic.
__device__ __forceinline__ void df_cell(df X, int nmax_cells, float& f, df& off) {
  float t = floorf(X.h);
  if (t == X.h && X.l < 0.f) t -= 1.f;                      // X just below an integer
  if (!(t >= 0.f)) t = 0.f;                                 // negative or NaN
  if (X.h < 0.f || (X.h == 0.f && X.l < 0.f)) X = {0.f, 0.f};
  if (t >= (float)nmax_cells) t = (float)(nmax_cells - 1);  // X itself is left unclamped (extrapolation)
  f = t;
  off = df_sub(X, {t, 0.f});
}

// Table-driven double-float log (Tang, "Table-driven implementation of the
// logarithm function in IEEE floating-point arithmetic", ACM TOMS 1990):
// entry j + 32 (j = -32..64) holds log c_j and 1 / c_j as float pairs for
// c_j = 1 + j / 128, filled on the host from FP64 values (upload_log_table).
constexpr int kLogTabLo = -32, kLogTabN = 97;
static __device__ float4 g_logtab[kLogTabN];

// log c_j + log1p(d / c_j) for |d / c_j| <= 2^-8 (d exact as a pair):
// log1p(u) = u - u^2/2 + u^3/3 in double-float and - u^4/4 + u^5/5 - u^6/6 +
// u^7/7 in FP32 (below 2^-34, the first omitted term below 2^-66).
__device__ __forceinline__ df df_log_core(int j, df d) {
  const float4 tb = __ldg(&g_logtab[j - kLogTabLo]);
  const df u = df_mul(d, df{tb.z, tb.w});
  const df u2 = df_mul(u, u);
  const df u3 = df_mul(u2, u);
  const float uh = u.h;
  const float tail = u2.h * u2.h * (-0.25f + uh * (0.2f - uh * (0.16666667f - uh * 0.14285715f)));
  const df third = {0x1.555556p-2f, -0x1.555556p-27f};
  df s = df_add(u, df{-0.5f * u2.h, -0.5f * u2.l});
  s = df_add(s, df_mul(u3, third));
  s.l += tail;
  return df_add(df{tb.x, tb.y}, s);
}

// log t for 2^-125 < t < 2^126: t = 2^k f with f in [0.75, 1.5) (so that t
// near 1 keeps k = 0: no cancellation of k ln 2 against log c), c = c_j the
// nearest table point, f - c exact (Sterbenz), log t = k ln 2 + log c +
// log1p((f - c) / c).  About 2^-47 relative.
__device__ __forceinline__ df df_log_tab(df t) {
  const int eb = (__float_as_int(t.h) >> 23) & 0xff;   // t.h = 1.m 2^(eb - 127), normal
  int k = eb - 127;
  const float sc = __int_as_float((254 - eb) << 23);   // 2^-k, exact
  df f = {t.h * sc, t.l * sc};                         // [1, 2)
  if (f.h >= 1.5f) {
    f = {0.5f * f.h, 0.5f * f.l};
    ++k;
  }
  int j = __float2int_rn((f.h - 1.f) * 128.f);
  j = min(max(j, kLogTabLo), kLogTabLo + kLogTabN - 1);
  const float c = __fmaf_rn((float)j, 0.0078125f, 1.f);   // 1 + j/128, exact
  df r = df_log_core(j, fast_two_sum(f.h - c, f.l));
  if (k != 0) r = df_add(df_scale(kDfLn2, (float)k), r);
  return r;
}

// log(1 + w) for -0.25 <= w < 0.5 without forming 1 + w: j = round(128 w),
// w - j/128 exact (Sterbenz for j != 0), log1p(w) = log c_j +
// log1p((w - j/128) / c_j).  About 2^-47 relative.
__device__ __forceinline__ df df_log1p_tab(df w) {
  int j = __float2int_rn(w.h * 128.f);
  j = min(max(j, kLogTabLo), kLogTabLo + kLogTabN - 1);
  return df_log_core(j, fast_two_sum(w.h - (float)j * 0.0078125f, w.l));
}

// asinh a for 0 <= a < 2^100: the series a (1 - a^2/6 + 3a^4/40 - 5a^6/112 +
// 35a^8/1152 - 63a^10/2816) below 1/16 (terms from a^6 in FP32, the first
// omitted below 2^-53); log1p(a + a^2 / (1 + sqrt(1 + a^2))) below 0.4 (w <
// 0.48: no rounding of 1 + w, which would cost up to 2^-44 relative near
// 1/16); log(a + sqrt(1 + a^2)) up to 2^24 (the result is above 0.39); log 2a
// above (the omitted 1/(4a^2) below 2^-50).
__device__ __forceinline__ df df_asinh_tab(df a) {
  const df one = {1.f, 0.f};
  if (a.h < 0.0625f) {
    const df a2 = df_mul(a, a);
    const float x = a2.h;
    const float tail = x * x * x * (-0.044642857f + x * (0.030381944f - x * 0.022372159f));
    const df sixth = {0x1.555556p-3f, -0x1.555556p-28f};
    const df c340 = {0x1.333334p-4f, -0x1.99999ap-29f};   // 3/40
    df p = df_add(one, df_neg(df_mul(a2, sixth)));
    p = df_add(p, df_mul(df_mul(a2, a2), c340));
    p.l += tail;
    return df_mul(a, p);
  }
  if (a.h < 0.4f) {
    const df a2 = df_mul(a, a);
    return df_log1p_tab(df_add(a, df_div(a2, df_add(one, df_sqrt(df_add(one, a2))))));
  }
  if (a.h < 16777216.f) return df_log_tab(df_add(a, df_sqrt(df_add(one, df_mul(a, a)))));
  return df_log_tab(df{2.f * a.h, 2.f * a.l});
}

// z / (|z| + eps) for the z map: +-(1 - delta) with delta = eps / (|z| + eps)
// in FP32 where delta < 2^-25 (then the pair is normalised and delta's FP32
// rounding is below 2^-49), the double-float quotient otherwise.
__device__ __forceinline__ df df_zsign(df z, df eps) {
  const float az = fabsf(z.h);
  if (az > eps.h * 33554432.f) {
    const float delta = __fdiv_rn(eps.h, az + eps.h);
    return z.h > 0.f ? df{1.f, -delta} : df{-1.f, delta};
  }
  return df_div(z, df_add(df_abs(z), eps));
}

static int upload_log_table() {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  XT_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(mu);
  if (dev >= 0 && dev < 64 && done[dev]) return XT_OK;
  float4 tab[kLogTabN];
  for (int i = 0; i < kLogTabN; ++i) {
    const double c = 1.0 + (i + kLogTabLo) / 128.0, L = std::log(c), inv = 1.0 / c;
    const float lh = (float)L, ih = (float)inv;
    tab[i] = make_float4(lh, (float)(L - (double)lh), ih, (float)(inv - (double)ih));
  }
  XT_CUDA(cudaMemcpyToSymbol(g_logtab, tab, sizeof(tab)));
  if (dev >= 0 && dev < 64) done[dev] = true;
  return XT_OK;
}

// The double-float functions of the FP64 binning on n values (diagnostics):
// fn 0 log x, 1 asinh x (x >= 0), 2 the z map z / (|z| + 1e-8) asinh |z|.
__global__ void k_df_eval(int fn, const double* __restrict__ in, double* __restrict__ out, long long n) {
  const df eps = df_from(1.0e-8);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const df x = df_from(in[i]);
    df r;
    if (fn == 0) r = df_log_tab(x);
    else if (fn == 1) r = df_asinh_tab(x);
    else r = df_mul(df_zsign(x, eps), df_asinh_tab(df_abs(x)));
    out[i] = df_to(r);
  }
}

// Table constants as float pairs, split on the host.
struct BinrecDf {
  df xmin, idx, ymin, idy, ias, ih, soft, zeps, m4pi;
};

static df host_df(double v) {
  const float h = (float)v;
  return {h, (float)(v - (double)h)};
}

__global__ void __launch_bounds__(256) k_cyl_binrec_df(CylTab<double> T, BinrecDf K, const double* __restrict__ x,
                                                       const double* __restrict__ y, const double* __restrict__ z,
                                                       const double* __restrict__ mass, long long n,
                                                       int* __restrict__ hist, BinRec<df>* __restrict__ rec,
                                                       double* __restrict__ Rout, int nan_to_origin,
                                                       double* __restrict__ zD, float* __restrict__ zE, long long nz,
                                                       int qchunk) {
  // zero the deposit grids (read by the deposit three kernels later)
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nz; i += (long long)gridDim.x * blockDim.x) {
    zD[i] = 0.0;
    zE[i] = 0.f;
  }
  const df xmin = K.xmin, idx = K.idx, ymin = K.ymin, idy = K.idy, ias = K.ias, one = {1.f, 0.f};
  const df soft = K.soft, zeps = K.zeps, m4pi = K.m4pi;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    double xx = x[p], yy = y[p], zz = z[p];
    if (nan_to_origin && (isnan(xx) || isnan(yy) || isnan(zz))) xx = yy = zz = 0.0;
    bool okx, oky, okz;
    const df xd = df_split(xx, okx), yd = df_split(yy, oky), zd = df_split(zz, okz);
    const df s2 = df_add(df_mul(xd, xd), df_mul(yd, yd));
    const bool safe = okx && oky && okz && fabsf(xd.h) < 1.0e15f && fabsf(yd.h) < 1.0e15f &&
                      fabsf(zd.h) < 1.0e15f && s2.h > 1.0e-30f;
    df dx, dy, c1, s1;
    float fx, fy;
    if (safe) {
      const df Rc = df_sqrt(df_add(s2, soft));
      const df irho = df_rsqrt(s2);               // cos, sin phi = x, y / rho
      c1 = df_mul(xd, irho);
      s1 = df_mul(yd, irho);
      df xi;
      if (T.cmap == 1) {
        const df u = df_mul(Rc, ias);
        xi = df_div(df_sub(u, one), df_add(u, one));
      } else if (T.cmap == 2) {
        xi = df_log_tab(Rc);
      } else {
        xi = Rc;
      }
      df_cell(df_mul(df_sub(xi, xmin), idx), T.numx, fx, dx);
      const df sg = df_zsign(zd, zeps);
      const df yv = df_mul(sg, df_asinh_tab(df_mul(df_abs(zd), K.ih)));
      df_cell(df_mul(df_sub(yv, ymin), idy), T.numy, fy, dy);
      if (Rout) Rout[p] = df_to_int(Rc);
    } else {
      const double Rd = sqrt(xx * xx + yy * yy + 1.0e-10);
      double c, s;
      unit_phi(xx, yy, c, s);
      c1 = df_from(c);
      s1 = df_from(s);
      double X = (r_to_xi_inv(Rd, T.cmap, T.inv_ascale) - T.XMIN) * T.inv_dX;
      double Y = (z_to_y_inv(zz, T.inv_hscale) - T.YMIN) * T.inv_dY;
      double tx = trunc(X), ty = trunc(Y);
      if (!(tx >= 0.0)) tx = 0.0;
      if (!(ty >= 0.0)) ty = 0.0;
      if (X < 0.0) X = 0.0;
      if (Y < 0.0) Y = 0.0;
      if (tx >= (double)T.numx) tx = (double)(T.numx - 1);
      if (ty >= (double)T.numy) ty = (double)(T.numy - 1);
      fx = (float)tx;
      fy = (float)ty;
      dx = df_from(X - tx);
      dy = df_from(Y - ty);
      if (Rout) Rout[p] = Rd;
    }
    const int ix = (int)fx, iy = (int)fy;
    BinRec<df> r;
    r.dx = dx;
    r.dy = dy;
    r.c1 = c1;
    r.s1 = s1;
    r.base = df_mul(df_split_or_from(mass[p]), m4pi);
    r.cell = ix * T.numy + iy;
    r.idx = atomicAdd(hist + sort_bucket(p, qchunk, T.numx * T.numy, r.cell), 1);
    rec[p] = r;
  }
}

// Exclusive prefix sum of hist[0..ncell) into off[] in two levels: tiles of
// 1024 cells scanned by one block each (warp shuffles), then the tile totals.
constexpr int kScanTile = 1024;

__device__ __forceinline__ int block_exclusive_scan_1024(int v, int* warp_tot, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int t = warp_tot[lane];
    int u = t;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, u, d);
      if (lane >= d) u += y;
    }
    warp_tot[lane] = u - t;           // exclusive prefix of warp totals
    if (lane == 31) warp_tot[32] = u;
  }
  __syncthreads();
  total = warp_tot[32];
  return x - v + warp_tot[wid];
}

// Node blocks of the tiled tables whose field the evaluation reads: those
// holding a corner node (ix + {0,1}, iy + {0,1}) of a cell with particles
// (cell = ix * numy + iy).  The deposit grid is zero outside them, so the
// contraction may skip the others as well.
struct ActiveBlocks {
  int* flag = nullptr;    // [nblk], cleared before the scan; nullptr: not wanted
  int* list = nullptr;    // [1 + nblk]: count, then the marked blocks in increasing order
  int numy = 0, ncell = 1, nblk = 0;   // the scanned counts are buckets (part, cell): cell = i % ncell
  TileOrder to{1, 1};
};

__global__ void __launch_bounds__(kScanTile) k_scan_tiles(const int* __restrict__ hist, int* __restrict__ off,
                                                          int* __restrict__ tile_sum, int ncell, ActiveBlocks ab) {
  __shared__ int wt[33];
  const int i = blockIdx.x * kScanTile + threadIdx.x;
  const int v = i < ncell ? hist[i] : 0;
  int total;
  const int ex = block_exclusive_scan_1024(v, wt, total);
  if (i < ncell) off[i] = ex;
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
  if (ab.flag && v > 0) {
    const int c = i % ab.ncell;
    const int ix = c / ab.numy, iy = c - ix * ab.numy;
    const size_t t00 = ab.to.pos(ix, iy), t01 = t00 + ab.to.nx1;   // (ix, iy + 1)
    ab.flag[t00 / kTileNodes] = 1;   // same-value stores: their order does not matter
    ab.flag[(t00 + 1) / kTileNodes] = 1;
    ab.flag[t01 / kTileNodes] = 1;
    ab.flag[(t01 + 1) / kTileNodes] = 1;
  }
}

// Adds the exclusive prefix of the tile totals (scanned by every block from
// the tile_sum array; ntile <= 1024) to each cell offset.  With ab.list, block
// 0 also lists the flagged node blocks in increasing order.
__global__ void __launch_bounds__(kScanTile) k_scan_add(int* __restrict__ off, const int* __restrict__ tile_sum,
                                                        int ncell, int ntile, ActiveBlocks ab) {
  __shared__ int wt[33];
  __shared__ int pref;
  const int t = threadIdx.x;
  int total;
  const int ex = block_exclusive_scan_1024(t < ntile ? tile_sum[t] : 0, wt, total);
  if (t == blockIdx.x) pref = ex;
  __syncthreads();
  const int i = blockIdx.x * kScanTile + t;
  if (i < ncell) off[i] += pref;
  if (ab.list && blockIdx.x == 0) {
    int base = 0;
    for (int b0 = 0; b0 < ab.nblk; b0 += kScanTile) {
      const int b = b0 + t;
      const int f = (b < ab.nblk && ab.flag[b]) ? 1 : 0;
      __syncthreads();   // wt is reused by consecutive scans
      const int at = block_exclusive_scan_1024(f, wt, total);
      if (f) ab.list[1 + base + at] = b;
      base += total;
    }
    if (t == 0) ab.list[0] = base;
  }
}

// Counting-sort scatter: record p moves to off[bucket] + its slot, carrying p.
// A thread takes kScatterUnroll records a grid stride apart at a time, so
// that their loads, the dependent offset loads and the scattered stores of
// several records are in flight together.
constexpr int kScatterUnroll = 4;

template <typename RT>
__global__ void __launch_bounds__(256) k_cyl_scatter(long long n, const int* __restrict__ off,
                                                     const BinRec<RT>* __restrict__ rec,
                                                     BinRec<RT>* __restrict__ srec, int qchunk, int ncell) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long p0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; p0 < n; p0 += kScatterUnroll * stride) {
    BinRec<RT> r[kScatterUnroll];
    long long q[kScatterUnroll];
#pragma unroll
    for (int u = 0; u < kScatterUnroll; ++u) {
      const long long p = p0 + u * stride;
      if (p < n) r[u] = rec[p];
    }
#pragma unroll
    for (int u = 0; u < kScatterUnroll; ++u) {
      const long long p = p0 + u * stride;
      if (p < n) q[u] = (long long)off[sort_bucket(p, qchunk, ncell, r[u].cell)] + r[u].idx;
    }
#pragma unroll
    for (int u = 0; u < kScatterUnroll; ++u) {
      const long long p = p0 + u * stride;
      if (p < n) {
        r[u].idx = (int)p;
        srec[q[u]] = r[u];
      }
    }
  }
}

// Evaluation of the binned records (accumulated_eval_particles outputs p0 p
// fr fp fz) numbered [*rbeg, *rend) (NULL: 0, n).  SORTED: records in bucket
// order with each result written back to the particle's original slot;
// otherwise the records in original order and coalesced result writes.
template <typename R, bool SORTED>
__global__ void __launch_bounds__(128) k_cyl_eval_sorted(CylTab<R> T, const R* __restrict__ F, long long n,
                                                         const BinRec<R>* __restrict__ recs, CylEvalOpts o,
                                                         double* o0, double* o1, double* o2, double* o3,
                                                         double* o4, const int* __restrict__ rbeg,
                                                         const int* __restrict__ rend) {
  const long long qb = rbeg ? *rbeg : 0, qe = rend ? *rend : n;
  for (long long q = qb + blockIdx.x * (long long)blockDim.x + threadIdx.x; q < qe;
       q += (long long)gridDim.x * blockDim.x) {
    const BinRec<R> r = recs[q];
    const int ix = r.cell / T.numy, iy = r.cell - ix * T.numy;
    CylBins<R> B;
    B.node = ix * (T.numy + 1) + iy;
    R w[4];
    weights_from_frac(r.dx, r.dy, w);
    B.c00 = w[0];
    B.c10 = w[1];
    B.c01 = w[2];
    B.c11 = w[3];
    R v[9];
    cyl_eval_bins(T, F, B, r.c1, r.s1, o, v);
    const long long p = SORTED ? (long long)r.idx : q;
    if (o0) o0[p] = v[0];
    if (o1) o1[p] = v[1];
    if (o2) o2[p] = v[2];
    if (o3) o3[p] = v[3];
    if (o4) o4[p] = v[4];
  }
}


__device__ __forceinline__ void df_weights(df dx, df dy, df w[4]) {
  const df one{1.f, 0.f};
  const df ex = df_sub(one, dx), ey = df_sub(one, dy);
  w[0] = df_mul(ex, ey);
  w[1] = df_mul(dx, ey);
  w[2] = df_mul(ex, dy);
  w[3] = df_mul(dx, dy);
}

// Arithmetic of the sorted deposit: FP32 sums (mixed path) or double-float
// sums (FP64 path), both widened to FP64 for the atomics.
// T is the record arithmetic, A the per-run sum (lazily renormalised for df).
struct DepF32 {
  using T = float;
  using A = float;
  static __device__ __forceinline__ T zero() { return 0.f; }
  static __device__ __forceinline__ T one() { return 1.f; }
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  static __device__ __forceinline__ A acc0() { return 0.f; }
  static __device__ __forceinline__ void acc(A& a, T x, T y) { a = x * y + a; }
  static __device__ __forceinline__ T twice(T c1) { return 2.f * c1; }
  static __device__ __forceinline__ T cheb(T c2, T cur, T prev) { return c2 * cur - prev; }   // c2 = 2 cos phi
  static __device__ __forceinline__ void weights(T dx, T dy, T w[4]) { weights_from_frac(dx, dy, w); }
  static __device__ __forceinline__ void deposit(double* D, float*, size_t i, A a) { atomicAdd(D + i, (double)a); }
  static __device__ __forceinline__ A merge(A a, A b) { return a + b; }
};
struct DepDF {
  using T = df;
  using A = dacc;
  static __device__ __forceinline__ T zero() { return df{0.f, 0.f}; }
  static __device__ __forceinline__ T one() { return df{1.f, 0.f}; }
  static __device__ __forceinline__ T mul(T a, T b) { return df_mul(a, b); }
  static __device__ __forceinline__ A acc0() { return dacc{}; }
  static __device__ __forceinline__ void acc(A& a, T x, T y) { a.fma(x, y); }
  static __device__ __forceinline__ T twice(T c1) { return df_scale(c1, 2.f); }   // exact
  static __device__ __forceinline__ T cheb(T c2, T cur, T prev) {   // c2 = 2 cos phi
    return df_sub(df_mul(c2, cur), prev);
  }
  static __device__ __forceinline__ void weights(T dx, T dy, T w[4]) { df_weights(dx, dy, w); }
  // leading part into the FP64 grid (one conversion, no FP64 add), the small
  // error part into the FP32 companion grid E (FP32 atomic); the contraction
  // reads D + E
  static __device__ __forceinline__ void deposit(double* D, float* E, size_t i, A a) {
    atomicAdd(D + i, (double)a.s);
    if (a.e != 0.f) atomicAdd(E + i, a.e);
  }
  // sum of two lazy sums: TwoSum of the leading parts, error parts added
  static __device__ __forceinline__ A merge(A a, A b) {
    const float t = __fadd_rn(a.s, b.s);
    const float v = __fsub_rn(t, a.s);
    const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, v)), __fsub_rn(b.s, v));
    A r;
    r.s = t;
    r.e = __fadd_rn(__fadd_rn(a.e, b.e), err);
    return r;
  }
};

// Lanes parked per cooperative flush batch: the whole warp, so that every
// same-cell run of a warp is added up before its atomics (measured on 1e6
// disc particles: FP64 deposit 0.110 / 0.103 / 0.100 ms with 8 / 16 / 32 slots,
// FP32 0.053 / 0.048 / 0.045 ms).
constexpr int kDepSlots = 32;

// Deposit of sorted records.  Each lane takes `run` consecutive particles and
// sums their contributions per (m, cos/sin, corner) in registers while the
// cell stays the same.  A lane whose cell changes (and every lane at the end
// of its run) parks its sums in shared memory; the whole warp then widens
// them to FP64 and issues the atomics, 32 entries per instruction.  (A
// divergent per-lane flush would occupy the FP64 unit for a full warp
// instruction per value however few lanes are active.)  Loops are
// warp-uniform so that the ballots see every lane.  With NPASS = 2 a run is
// deposited in two passes over its records, the cosine sums (m = 0..MCAP)
// and then the sine sums (m = 1..MCAP), so that half the sums are live at a
// time (double-float sums: 104 -> 56 registers of accumulators, for more
// resident warps) and each pass runs only its own Chebyshev recurrence; the
// second pass re-reads the run's records from L1.  The grids D and E are
// indexed by the tile position of the node (TileOrder: rows of constant z),
// the order in which the contraction reads them.
template <typename M, int MCAP, int NPASS>
__global__ void __launch_bounds__(128, NPASS == 2 ? 4 : (MCAP <= 6 ? 3 : 2))
    k_cyl_deposit_sorted(int numy, int nx1, int mmax, long long n, int run,
                         const BinRec<typename M::T>* __restrict__ srec, double* __restrict__ D,
                         float* __restrict__ E, size_t plane) {
  using T = typename M::T;
  using A = typename M::A;
  // sums per pass: all 2 MCAP + 1 in one pass, else the cosines then the sines
  constexpr int NJ0 = NPASS == 2 ? MCAP + 1 : 2 * MCAP + 1, NJ1 = MCAP;
  constexpr int NEMAX = 4 * (NJ0 > NJ1 ? NJ0 : NJ1);
  constexpr int PITCH = NEMAX + 1;              // conflict-free parking of up to 8 lanes
  __shared__ A park[4][kDepSlots][PITCH];
  __shared__ int park_node[4][kDepSlots];     // tile position of the parked lane's lower-left node
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int nju = 2 * mmax + 1;                 // sums in use (global index j)
  const long long nrun = (n + run - 1) / run;

  auto run_pass = [&](long long q0, auto pass_tag) {
    constexpr int PASS = decltype(pass_tag)::value;
    constexpr bool COS = NPASS == 1 || PASS == 0, SIN = NPASS == 1 || PASS == 1;
    constexpr int NJP = PASS == 0 ? NJ0 : NJ1;
    // global sum index j (0: m = 0 cosine; 2m - 1: cosine m; 2m: sine m) of
    // this pass's local index jl
    auto gj = [](int jl) { return NPASS == 1 ? jl : (PASS == 0 ? (jl ? 2 * jl - 1 : 0) : 2 * (jl + 1)); };
    constexpr int NE = 4 * NJP;
    A acc[NJP][4];
#pragma unroll
    for (int j = 0; j < NJP; ++j)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[j][k] = M::acc0();
    // park the sums of the lanes in `want`, batch by batch, and deposit them
    auto flush = [&](bool want, int cell) {
      unsigned pend = __ballot_sync(0xffffffffu, want);
      while (pend) {
        unsigned batch = 0, rest = pend;
        for (int i = 0; i < kDepSlots && rest; ++i) {
          batch |= rest & (0u - rest);
          rest &= rest - 1;
        }
        const int nb = __popc(batch);
        if (batch & (1u << lane)) {
          const int sidx = __popc(batch & ((1u << lane) - 1));
          const int ix = cell / numy, iy = cell - ix * numy;
          park_node[wib][sidx] = iy * nx1 + ix;
#pragma unroll
          for (int j = 0; j < NJP; ++j)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              park[wib][sidx][j * 4 + k] = acc[j][k];
              acc[j][k] = M::acc0();
            }
        }
        __syncwarp();
        // one lane per sum entry e across the batch's slots; slots of the same
        // cell (adjacent, as the runs are in cell order) are added before
        // their atomics
        for (int e = lane; e < NE; e += 32) {
          const int j = gj(e >> 2), k = e & 3;
          if (j < nju) {
            const int m = (j + 1) >> 1;        // j = 0: m=0 cos; j = 2m-1: cos m; j = 2m: sin m
            const int cs = (j != 0 && !(j & 1)) ? 1 : 0;
            const size_t off = (size_t)(2 * m + cs) * plane + ((k & 1) ? 1 : 0) + ((k & 2) ? nx1 : 0);
            int nd = park_node[wib][0];
            A a = park[wib][0][e];
            for (int sidx = 1; sidx < nb; ++sidx) {
              const int nd2 = park_node[wib][sidx];
              const A b = park[wib][sidx][e];
              if (nd2 == nd) {
                a = M::merge(a, b);
              } else {
                M::deposit(D, E, off + nd, a);
                nd = nd2;
                a = b;
              }
            }
            M::deposit(D, E, off + nd, a);
          }
        }
        __syncwarp();
        pend &= ~batch;
      }
    };
    int cur = -1;
#pragma unroll 1
    for (int u = 0; u < run; ++u) {
      const long long q = q0 + u;
      const bool valid = q < n;                 // also false for lanes past the last run
      BinRec<T> r;
      if (valid) r = srec[q];
      const int c = valid ? r.cell : cur;
      flush(cur >= 0 && c != cur, cur);
      cur = c;
      if (!valid) continue;
      T w[4];
      M::weights(r.dx, r.dy, w);
      const T c1 = r.c1, s1 = r.s1, base = r.base, c2 = M::twice(c1);
      T cprev = M::one(), sprev = M::zero(), ccur = c1, scur = s1;
#pragma unroll
      for (int m = 0; m <= MCAP; ++m) {
        if (m > mmax) break;
        T cm, sm;
        if (m == 0) { cm = M::one(); sm = M::zero(); }
        else if (m == 1) { cm = c1; sm = s1; }
        else {
          if constexpr (COS) { cm = M::cheb(c2, ccur, cprev); cprev = ccur; ccur = cm; }
          if constexpr (SIN) { sm = M::cheb(c2, scur, sprev); sprev = scur; scur = sm; }
        }
        if constexpr (COS) {
          const T wc = M::mul(base, cm);
          const int jc = NPASS == 1 ? ((m == 0) ? 0 : 2 * m - 1) : m;
#pragma unroll
          for (int k = 0; k < 4; ++k) M::acc(acc[jc][k], wc, w[k]);
        }
        if constexpr (SIN) {
          if (m > 0) {
            const T ws = M::mul(base, sm);
            const int js = NPASS == 1 ? 2 * m : m - 1;
#pragma unroll
            for (int k = 0; k < 4; ++k) M::acc(acc[js][k], ws, w[k]);
          }
        }
      }
    }
    flush(cur >= 0, cur);
  };

  for (long long r0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); r0 < nrun;
       r0 += (long long)gridDim.x * blockDim.x) {
    const long long q0 = (r0 + lane) * run;
    run_pass(q0, std::integral_constant<int, 0>{});
    if constexpr (NPASS == 2) {
      if (mmax > 0) run_pass(q0, std::integral_constant<int, 1>{});
    }
  }
}

template <typename OT>
__device__ __forceinline__ OT from_df(df v);
template <>
__device__ __forceinline__ df from_df<df>(df v) { return v; }
template <>
__device__ __forceinline__ float from_df<float>(df v) { return v.h + v.l; }

// Field of the fused paths: coefficients staged in shared memory as df,
// lazily renormalised df sums on the FP32 pipe (no FP64 pipe work at all).
// SPLIT: double-float tables (tiled FP32 roundings + 16-bit remainders) and
// a df field (FP64 path); otherwise the tiled FP32 roundings alone and an
// FP32 field (mixed path).  Block b owns node block b of the tiled tables
// (kTileNodes nodes, one contiguous region of them).  Each thread computes
// one (m, field) entry for a quad of consecutive nodes from 16-byte loads of
// hi and 8-byte loads of the remainders, RB table rows in flight and four
// independent sums.  The block's nodes are written back through shared
// memory, each node's entries contiguous, in the layout of k_cyl_field with
// nf = 6.  Block i takes the node block blist[1 + i] of the blist[0] listed;
// the field of the others is not written.
template <typename OT, bool SPLIT, int RB, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) k_cyl_field2(const float* __restrict__ hi, const short* __restrict__ lo,
                                                    const double* __restrict__ cosc, const double* __restrict__ sinc,
                                                    int mmax, int norder, size_t nnode, TileOrder to,
                                                    const int* __restrict__ blist, OT* __restrict__ F) {
  constexpr int QN = kTileNodes, TQ = QN / 4;
  if ((int)blockIdx.x >= blist[0]) return;   // blocks past the listed node blocks
  const size_t bid = (size_t)blist[1 + blockIdx.x];
  extern __shared__ unsigned char smem_raw[];
  df* cf = reinterpret_cast<df*>(smem_raw);                       // [2][(mmax+1)*norder]
  OT* tile = reinterpret_cast<OT*>(cf + 2 * (mmax + 1) * norder);
  const int ncoef = (mmax + 1) * norder;
  for (int i = threadIdx.x; i < 2 * ncoef; i += blockDim.x) cf[i] = df_from(i < ncoef ? cosc[i] : sinc[i - ncoef]);
  __syncthreads();
  const int nf = 6;
  const int mf_total = (mmax + 1) * nf;
  const size_t node0 = bid * QN;
  const size_t tbase = bid * 6 * ncoef * QN;
  for (int task = threadIdx.x; task < TQ * mf_total; task += blockDim.x) {
    const int ql = task % TQ;
    const int mf = task / TQ;
    const int m = mf / nf, f = mf % nf;
    dacc acc[4];
    if (node0 + 4 * ql < nnode && !(m == 0 && f >= 3)) {
      const df* coef = cf + ((f >= 3) ? ncoef : 0) + m * norder;
      const size_t t0 = tbase + (size_t)(f * ncoef + m * norder) * QN + 4 * ql;
      for (int k0 = 0; k0 < norder; k0 += RB) {
        float4 vh[RB];
        short4 vl[RB];
#pragma unroll
        for (int u = 0; u < RB; ++u) {
          if (k0 + u < norder) {
            vh[u] = *reinterpret_cast<const float4*>(hi + t0 + (size_t)(k0 + u) * QN);
            vl[u] = SPLIT ? *reinterpret_cast<const short4*>(lo + t0 + (size_t)(k0 + u) * QN)
                          : make_short4(0, 0, 0, 0);
          }
        }
#pragma unroll
        for (int u = 0; u < RB; ++u) {
          if (k0 + u < norder) {
            const df c = coef[k0 + u];
            if constexpr (SPLIT) {
              const float cs = c.h * kLo16Scale;
              acc[0].fma_lo16(c, cs, vh[u].x, lo16_unscaled(vh[u].x, vl[u].x));
              acc[1].fma_lo16(c, cs, vh[u].y, lo16_unscaled(vh[u].y, vl[u].y));
              acc[2].fma_lo16(c, cs, vh[u].z, lo16_unscaled(vh[u].z, vl[u].z));
              acc[3].fma_lo16(c, cs, vh[u].w, lo16_unscaled(vh[u].w, vl[u].w));
            } else {
              acc[0].fma(c, df{vh[u].x, 0.f});
              acc[1].fma(c, df{vh[u].y, 0.f});
              acc[2].fma(c, df{vh[u].z, 0.f});
              acc[3].fma(c, df{vh[u].w, 0.f});
            }
          }
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) tile[(4 * ql + j) * mf_total + mf] = from_df<OT>(acc[j].value());
  }
  __syncthreads();
  const size_t nvalid = (node0 + QN <= nnode) ? QN : (nnode - node0);
  for (int idx = threadIdx.x; idx < (int)(nvalid * mf_total); idx += blockDim.x) {
    const int j = idx / mf_total;
    F[to.node(node0 + j) * mf_total + (idx - j * mf_total)] = tile[idx];
  }
}

// Field of the fused paths through a bulk-copy (TMA) pipeline.  The work is
// cut into units of (listed node block, field f, m-range of mg values of m);
// persistent CTA c takes the units [c U / G, (c + 1) U / G) of the U in
// order (G CTAs).  The table rows of a unit are one contiguous run of the
// tiled tables (rows (f, m, k) for m in the range, every k; for the sine
// fields the m = 0 rows are skipped), which the copy warp moves into a ring of
// nstage shared-memory stages with cp.async.bulk, counted on the stage's
// `full` mbarrier.  Two groups of fourteen compute warps take alternate
// units, so that two units are summed while the next are in flight.  In a
// group, warp-task (m, half) covers 16 node pairs; lane (k half, pair) sums
// its half of the orders for both nodes of its pair in lazily renormalised
// double-float, one shuffle joins the halves (the lane of the first half
// keeps the even position, the other the odd), and the lane stores its node's
// entry of F (layout of k_cyl_field with nf = 6; the m = 0 sine entries are
// written as zero).  A group's warps release the stage on its `empty`
// mbarrier; the copy warp refills it.  Waits are bounded: a timeout sets
// *err = 1 and an abort flag that ends every later wait at once; the copy
// warp stops issuing, and waits (bounded) for its copies in flight before it
// exits.
constexpr int kFieldGroupWarps = 14;
constexpr int kFieldComputeWarps = 2 * kFieldGroupWarps;
constexpr int kFieldThreads = 32 * (kFieldComputeWarps + 1);
constexpr int kFieldMaxStages = 8;

__device__ __forceinline__ bool field_wait(uint32_t addr, uint32_t parity, volatile int* abort, int* err) {
  for (long long it = 0; it < TC_SPIN_LIMIT; ++it) {
    if (mbar_test(addr, parity)) return true;
    if (*abort) return false;
  }
  *abort = 1;
  atomicExch(err, 1);
  return false;
}

template <typename OT, bool SPLIT>
__global__ void __launch_bounds__(kFieldThreads, 1)
    k_cyl_field_bulk(const float* __restrict__ hi, const short* __restrict__ lo, const double* __restrict__ cosc,
                     const double* __restrict__ sinc, int mmax, int norder, size_t nnode, TileOrder to,
                     const int* __restrict__ blist, int mg, int nstage, unsigned stage_hi_bytes,
                     unsigned stage_bytes, unsigned cf_bytes, OT* __restrict__ F, int* __restrict__ err) {
  constexpr int QN = kTileNodes;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ int s_abort;
  const int ncoef = (mmax + 1) * norder;
  const int mf_total = (mmax + 1) * 6;
  const int nmc = (mmax + mg) / mg;
  const int per_block = 6 * nmc;
  const long long ntot = (long long)blist[0] * per_block;
  const int u0 = (int)(ntot * blockIdx.x / gridDim.x);
  const int nunit = (int)(ntot * (blockIdx.x + 1) / gridDim.x) - u0;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
  uint64_t* empty = full + kFieldMaxStages;
  df* cf = reinterpret_cast<df*>(smem_raw + 128);
  unsigned char* stages = smem_raw + 128 + cf_bytes;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    s_abort = 0;
    for (int i = 0; i < nstage; ++i) {
      mbar_init_count(smem_u32(full + i), 1);
      mbar_init_count(smem_u32(empty + i), kFieldGroupWarps);
    }
    mbar_init_fence();
  }
  for (int i = threadIdx.x; i < 2 * ncoef; i += blockDim.x) cf[i] = df_from(i < ncoef ? cosc[i] : sinc[i - ncoef]);
  __syncthreads();
  volatile int* abort = &s_abort;
  // unit u: node block b, field f, m in [ma, mb); rows copied from m = mc0
  // (ma, or 1 for the sine fields when ma = 0)
  auto unit = [&](int u, int& b, int& f, int& ma, int& mc0, int& mb) {
    const int j = u / per_block, r = u - j * per_block;
    f = r / nmc;
    ma = (r - f * nmc) * mg;
    mb = min(mmax + 1, ma + mg);
    mc0 = (f >= 3 && ma == 0) ? 1 : ma;
    b = blist[1 + j];
  };

  if (warp == kFieldComputeWarps) {
    // copy warp: one lane issues every unit's copies
    if (lane != 0) return;
    int issued = 0;
    for (int v = 0; v < nunit; ++v) {
      const int st = v % nstage, use = v / nstage;
      if (use > 0 && !field_wait(smem_u32(empty + st), (use - 1) & 1, abort, err)) break;
      int b, f, ma, mc0, mb;
      unit(u0 + v, b, f, ma, mc0, mb);
      const uint32_t fa = smem_u32(full + st);
      const unsigned rows = mb > mc0 ? (unsigned)((mb - mc0) * norder) : 0u;
      if (rows == 0) {
        mbar_arrive(fa);
      } else {
        const unsigned bh = rows * QN * 4u, bl = SPLIT ? rows * QN * 2u : 0u;
        const size_t src = (size_t)b * 6 * ncoef * QN + ((size_t)f * ncoef + (size_t)mc0 * norder) * QN;
        mbar_arrive_expect_tx(fa, bh + bl);
        bulk_load(smem_u32(stages + (size_t)st * stage_bytes), hi + src, bh, fa);
        if (SPLIT) bulk_load(smem_u32(stages + (size_t)st * stage_bytes + stage_hi_bytes), lo + src, bl, fa);
      }
      issued = v + 1;
    }
    // the copies still in flight land before the CTA may end
    for (int v = max(0, issued - nstage); v < issued; ++v) mbar_wait(smem_u32(full + v % nstage), (v / nstage) & 1);
    return;
  }

  const int group = warp / kFieldGroupWarps, gw = warp - group * kFieldGroupWarps;
  const int kh = lane >> 4, p16 = lane & 15;
  const int khalf = (norder + 1) >> 1;
  const int kb = kh ? khalf : 0, ke = kh ? norder : khalf;
  for (int v = group; v < nunit; v += 2) {
    const int st = v % nstage;
    field_wait(smem_u32(full + st), (v / nstage) & 1, abort, err);
    int b, f, ma, mc0, mb;
    unit(u0 + v, b, f, ma, mc0, mb);
    const float* sh = reinterpret_cast<const float*>(stages + (size_t)st * stage_bytes);
    const short* sl = reinterpret_cast<const short*>(stages + (size_t)st * stage_bytes + stage_hi_bytes);
    const df* c0 = cf + (f >= 3 ? ncoef : 0);
    const size_t t0 = (size_t)b * QN;   // the block's first tile position
    const int iy0 = (int)(t0 / to.nx1), ix0 = (int)(t0 - (size_t)iy0 * to.nx1);
    for (int wt = gw; wt < 2 * (mb - ma); wt += kFieldGroupWarps) {
      const int m = ma + (wt >> 1);
      const int p = ((wt & 1) << 4) | p16;
      dacc a0, a1;
      if (m >= mc0) {
        const size_t row0 = (size_t)(m - mc0) * norder * QN + 2 * p;
        const df* c = c0 + m * norder;
#pragma unroll 3
        for (int k = kb; k < ke; ++k) {
          const float2 h = *reinterpret_cast<const float2*>(sh + row0 + (size_t)k * QN);
          const df ck = c[k];
          if constexpr (SPLIT) {
            const short2 l = *reinterpret_cast<const short2*>(sl + row0 + (size_t)k * QN);
            const float cks = ck.h * kLo16Scale;
            a0.fma_lo16(ck, cks, h.x, lo16_unscaled(h.x, l.x));
            a1.fma_lo16(ck, cks, h.y, lo16_unscaled(h.y, l.y));
          } else {
            a0.fma(ck, df{h.x, 0.f});
            a1.fma(ck, df{h.y, 0.f});
          }
        }
      }
      // the first k half keeps node 2p, the second node 2p + 1
      const df send = kh ? a0.raw() : a1.raw();
      const df own = kh ? a1.raw() : a0.raw();
      const df recv = {__shfl_xor_sync(0xffffffffu, send.h, 16), __shfl_xor_sync(0xffffffffu, send.l, 16)};
      const int o = 2 * p + kh;   // offset in the block: position t0 + o, node (ix, iy)
      if (t0 + o < nnode) {
        int ix = ix0 + o, iy = iy0;
        while (ix >= to.nx1) {   // at most 64 / nx1 + 1 rows
          ix -= to.nx1;
          ++iy;
        }
        F[((size_t)ix * to.ny1 + iy) * mf_total + m * 6 + f] = from_df<OT>(df_add(own, recv));
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(smem_u32(empty + st));
  }
}

// Field engine of the fused paths: 0 chooses the bulk-copy pipeline where its
// stages fit in shared memory, 1 requires it, 2 uses the row-load kernel.
static int g_field_engine = 0;
static __device__ int g_cyl_err;

// Shared-memory plan of k_cyl_field_bulk: the widest m-range (mg) whose
// stages fit four deep (one summed by each compute group, two in flight)
// beside the coefficients, and as many stages (up to kFieldMaxStages) as then
// fit.
struct FieldBulkPlan {
  int mg = 0, nstage = 0;
  unsigned stage_hi = 0, stage = 0, cf = 0;
  size_t smem = 0;
};

static bool field_bulk_plan(const CylHandle* h, bool f64, FieldBulkPlan& P) {
  static int optin = -1;
  if (optin < 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
      optin = 0;
  }
  const size_t cap = optin > 1024 ? (size_t)optin - 1024 : 0;   // 1 KB for the static shared variables
  const size_t ncoef = (size_t)(h->mmax + 1) * h->norder;
  P.cf = (unsigned)((2 * ncoef * sizeof(df) + 127) & ~(size_t)127);
  const size_t fixed = 128 + P.cf;
  for (int mg = h->mmax + 1; mg >= 1; --mg) {
    const size_t shi = (size_t)mg * h->norder * kTileNodes * sizeof(float);
    const size_t st = shi + (f64 ? (size_t)mg * h->norder * kTileNodes * sizeof(short) : 0);
    if (fixed + 4 * st <= cap) {
      P.mg = mg;
      P.nstage = (int)std::min<size_t>(kFieldMaxStages, (cap - fixed) / st);
      P.stage_hi = (unsigned)shi;
      P.stage = (unsigned)st;
      P.smem = fixed + (size_t)P.nstage * st;
      return true;
    }
  }
  return false;
}

// Double-float evaluation of the binned records (FP64 path,
// accumulated_eval_particles); SORTED and the record range [*rbeg, *rend)
// (NULL: 0, n) as for k_cyl_eval_sorted.
// Launch bounds and the twice-unrolled m loop were measured on 1e6 disc
// particles: 0.129 ms with up to ~127 registers, against 0.135 ms at 72;
// asking for 5 resident blocks (at most 102 registers) gives 0.121 ms, 6
// blocks or a rolled m loop 0.127 ms.  Two threads per record (orders split
// between the lanes of a pair, sums exchanged by shuffles; 64 registers, twice
// the warps) took 0.152 ms: the kernel is bound by its double-float
// instruction count, not by latency.  Interpolation sums split against a
// power of two above the cell's partial sums (ExtractScalar: 7 FP32
// operations a product instead of 12) took 0.1136 ms against 0.1165, with
// spills at 96 registers and about 3x the interpolation's rounding error: not
// taken.
template <bool SORTED>
__global__ void __launch_bounds__(128, 5) k_cyl_eval_sorted_df(CylTab<double> T, const df* __restrict__ F, long long n,
                                                            const BinRec<df>* __restrict__ recs, int m1, int m2,
                                                            double* o0, double* o1, double* o2, double* o3,
                                                            double* o4, const int* __restrict__ rbeg,
                                                            const int* __restrict__ rend) {
  const int ny1 = T.numy + 1;
  const int stride = (T.mmax + 1) * 6;
  const long long qb = rbeg ? *rbeg : 0, qe = rend ? *rend : n;
  for (long long q = qb + blockIdx.x * (long long)blockDim.x + threadIdx.x; q < qe;
       q += (long long)gridDim.x * blockDim.x) {
    const BinRec<df> r = recs[q];
    const int ix = r.cell / T.numy, iy = r.cell - ix * T.numy;
    const df* f00 = F + (size_t)(ix * ny1 + iy) * stride;
    const df* f01 = f00 + stride;
    const df* f10 = f00 + (size_t)ny1 * stride;
    const df* f11 = f10 + stride;
    df w[4];
    df_weights(r.dx, r.dy, w);
    const df w0 = w[0], w1 = w[1], w2 = w[2], w3 = w[3];
    const df c1 = r.c1, s1 = r.s1, c2 = df_scale(c1, 2.f);   // c2: exact
    // bilinear interpolation of the six fields of order m (lazy df sums, read
    // unnormalised by the products that follow).  A corner's six fields of
    // one m are 48 contiguous bytes at a 16-byte boundary (nodes 336 bytes
    // apart): three 16-byte loads, taken corner by corner.
    auto ld6 = [](const df* p, df f[6]) {
      const float4* q = reinterpret_cast<const float4*>(p);
      const float4 a = q[0], b = q[1], c = q[2];
      f[0] = {a.x, a.y};
      f[1] = {a.z, a.w};
      f[2] = {b.x, b.y};
      f[3] = {b.z, b.w};
      f[4] = {c.x, c.y};
      f[5] = {c.z, c.w};
    };
    auto interp = [&](int m, df v[6]) {
      const int b = m * 6;
      dacc a[6];
      df f[6];
      ld6(f00 + b, f);
#pragma unroll
      for (int k = 0; k < 6; ++k) a[k].set(f[k], w0);
      ld6(f10 + b, f);
#pragma unroll
      for (int k = 0; k < 6; ++k) a[k].fma(f[k], w1);
      ld6(f01 + b, f);
#pragma unroll
      for (int k = 0; k < 6; ++k) a[k].fma(f[k], w2);
      ld6(f11 + b, f);
#pragma unroll
      for (int k = 0; k < 6; ++k) a[k].fma(f[k], w3);
#pragma unroll
      for (int k = 0; k < 6; ++k) v[k] = a[k].raw();
    };
    df p0{0.f, 0.f};
    dacc p, fr, fp, fz;
    if (m1 <= 0 && m2 >= 0) {                   // m = 0: cos 0 = 1, sin 0 = 0
      df v[3];                                  // the sine fields of m = 0 are zero
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        dacc a;
        a.set(f00[k], w0);
        a.fma(f10[k], w1);
        a.fma(f01[k], w2);
        a.fma(f11[k], w3);
        v[k] = a.raw();
      }
      p0 = v[0];
      fr.s = v[1].h; fr.e = v[1].l;
      fz.s = v[2].h; fz.e = v[2].l;
    }
    df cprev{1.f, 0.f}, sprev{0.f, 0.f}, ccur = c1, scur = s1;
#pragma unroll 2
    for (int m = 1; m <= T.mmax; ++m) {
      df cm, sm;
      if (m == 1) { cm = c1; sm = s1; }
      else {
        cm = df_sub(df_mul(c2, ccur), cprev);
        sm = df_sub(df_mul(c2, scur), sprev);
        cprev = ccur; sprev = scur; ccur = cm; scur = sm;
      }
      if (m < m1 || m > m2) continue;
      df v[6];
      interp(m, v);
      p.fma(cm, v[0]);
      p.fma(sm, v[3]);
      fr.fma(cm, v[1]);
      fr.fma(sm, v[4]);
      fz.fma(cm, v[2]);
      fz.fma(sm, v[5]);
      fp.fma(df_scale(sm, (float)m), v[0]);     // m (sin(m phi) v0 - cos(m phi) v3)
      fp.fma(df_neg(df_scale(cm, (float)m)), v[3]);
    }
    const long long pidx = SORTED ? (long long)r.idx : q;
    if (o0) o0[pidx] = df_to(p0);
    if (o1) o1[pidx] = df_to(p.raw());
    if (o2) o2[pidx] = df_to(fr.raw());
    if (o3) o3[pidx] = df_to(fp.raw());
    if (o4) o4[pidx] = df_to(fz.raw());
  }
}

static const int kContractChunks = 8;
static const int kContractChunksDf = 64;   // most node chunks of k_cyl_contract_df
static const int kContractRows = 6;        // orders k per k_cyl_contract_df block

// Coefficient contraction of the fused paths:
//   cos/sin[m][k] = sum over nodes of (D + E)[2m+cs][node] * pot{C,S}[m][k][node]
// (E: the FP32 companion grid of the double-float deposit's error parts).
// Block (x = chunk * ngroup + g, y = p) takes a range of node quads of the
// (m, cs) pair p (0: m = 0 cosine; 2m - 1, 2m: m >= 1 cosine, sine; the m = 0
// sine is identically zero and has no block) for the KB orders k of group g.
// Each thread multiplies the quads' FP64 sums (split into float pairs by
// integer operations) by the tiled double-float tables (16-byte loads of hi,
// 8-byte loads of the 16-bit remainders, all KB rows in flight) in lazily
// renormalised df sums; a quad is four consecutive tile positions, and D and
// E are indexed by tile position as well.  The groups of one chunk are neighbouring blocks, so
// D and E are read once from DRAM.  The block's sums are reduced in df (warp
// shuffles, then shared memory) and stored per chunk as FP64 for
// k_cyl_contract_final.  D planes have a pitch of `pitch` nodes; padding
// entries are zero in D and in the tiled tables.  Only the node blocks of
// blist (count, then block indices) are read: D is zero in the others.
template <int KB>
__global__ void __launch_bounds__(128) k_cyl_contract_df(const float* __restrict__ hi, const short* __restrict__ lo,
                                                         size_t pitch, const double* __restrict__ D,
                                                         const float* __restrict__ E, int mmax, int norder,
                                                         size_t nnode, int nchunk, int ngroup,
                                                         const int* __restrict__ blist, double* __restrict__ part) {
  const int chunk = blockIdx.x / ngroup, g = blockIdx.x - chunk * ngroup, p = blockIdx.y;
  const int m = (p + 1) >> 1, cs = p ? ((p + 1) & 1) : 0;
  const int kbase = g * KB;
  dacc acc[KB];
  {
    constexpr int QB = kTileNodes / 4;   // quads per node block
    const int nq = blist[0] * QB;
    const int per = (nq + nchunk - 1) / nchunk;
    const int q0 = chunk * per, q1 = min(q0 + per, nq);
    const size_t nrow = 6 * (size_t)(mmax + 1) * norder;
    const size_t row0 = ((size_t)(cs ? 3 : 0) * (mmax + 1) + m) * norder + kbase;
    const double* d = D + (size_t)(2 * m + cs) * pitch;
    const float* ep = E + (size_t)(2 * m + cs) * pitch;
    for (int q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
      const size_t blk = (size_t)blist[1 + q / QB];
      const size_t t = blk * kTileNodes + 4 * (q % QB);   // tile position of the quad's first node
      if (t >= nnode) continue;   // past the last node (pitch: nnode rounded up to 4; D, E zero there)
      const size_t tb = (blk * nrow + row0) * kTileNodes + t % kTileNodes;
      float4 vh[KB];
      short4 vl[KB];
#pragma unroll
      for (int u = 0; u < KB; ++u) {
        if (kbase + u < norder) {
          const size_t o = tb + (size_t)u * kTileNodes;
          vh[u] = *reinterpret_cast<const float4*>(hi + o);
          vl[u] = *reinterpret_cast<const short4*>(lo + o);
        }
      }
      const double2 da = *reinterpret_cast<const double2*>(d + t);
      const double2 db = *reinterpret_cast<const double2*>(d + t + 2);
      const float4 ev = *reinterpret_cast<const float4*>(ep + t);
      const df dv[4] = {df_add(df_split_or_from(da.x), {ev.x, 0.f}), df_add(df_split_or_from(da.y), {ev.y, 0.f}),
                        df_add(df_split_or_from(db.x), {ev.z, 0.f}), df_add(df_split_or_from(db.y), {ev.w, 0.f})};
      const float dvs[4] = {dv[0].h * kLo16Scale, dv[1].h * kLo16Scale, dv[2].h * kLo16Scale, dv[3].h * kLo16Scale};
#pragma unroll
      for (int u = 0; u < KB; ++u) {
        if (kbase + u < norder) {
          acc[u].fma_lo16(dv[0], dvs[0], vh[u].x, lo16_unscaled(vh[u].x, vl[u].x));
          acc[u].fma_lo16(dv[1], dvs[1], vh[u].y, lo16_unscaled(vh[u].y, vl[u].y));
          acc[u].fma_lo16(dv[2], dvs[2], vh[u].z, lo16_unscaled(vh[u].z, vl[u].z));
          acc[u].fma_lo16(dv[3], dvs[3], vh[u].w, lo16_unscaled(vh[u].w, vl[u].w));
        }
      }
    }
  }
  __shared__ df red[4][KB];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int u = 0; u < KB; ++u) {
    df v = acc[u].value();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const df w{__shfl_down_sync(0xffffffffu, v.h, o), __shfl_down_sync(0xffffffffu, v.l, o)};
      v = df_add(v, w);
    }
    if (lane == 0) red[wid][u] = v;
  }
  __syncthreads();
  if (threadIdx.x < KB && kbase + (int)threadIdx.x < norder) {
    const int u = threadIdx.x, k = kbase + u;
    df v = red[0][u];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = df_add(v, red[w][u]);
    part[((size_t)(m * norder + k) * 2 + cs) * nchunk + chunk] = df_to(v);
  }
}

bool cyl_tabs(void* handle, CylTab<double>* d, CylTab<float>* f) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  if (!h) return false;
  if (d) *d = h->tab_d;
  if (f) *f = h->tab_f;
  return true;
}

// Exclusive scan of ncell (<= 1024^2) counts into off (may equal hist), with
// a scratch of 1024 ints: per-tile scans, then the tiles' prefix (also used by
// the orbit reordering).
int launch_cell_scan(const int* hist, int* off, int* tile_sum, int ncell, cudaStream_t st) {
  XT_REQUIRE(ncell >= 1 && ncell <= kScanTile * kScanTile, "scan of %d cells", ncell);
  const int ntile = (ncell + kScanTile - 1) / kScanTile;
  k_scan_tiles<<<ntile, kScanTile, 0, st>>>(hist, off, tile_sum, ncell, ActiveBlocks{});
  XT_CHECK_LAUNCH("k_scan_tiles");
  k_scan_add<<<ntile, kScanTile, 0, st>>>(off, tile_sum, ncell, ntile, ActiveBlocks{});
  XT_CHECK_LAUNCH("k_scan_add");
  return XT_OK;
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
  if (int rc = upload_log_table()) return rc;   // the binning's log table
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
  if (cudaStreamCreateWithFlags(&h->copy, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->qdone, cudaEventDisableTiming) != cudaSuccess) {
    xt_cyl_table_destroy(h);
    return cuda_fail(cudaGetLastError(), "copy stream / events");
  }
  for (cudaEvent_t& ev : h->qev)
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
      xt_cyl_table_destroy(h);
      return cuda_fail(cudaGetLastError(), "copy events");
    }
  h->tab_d = CylTab<double>{mmax, norder, numx, numy, cmap, XMIN, dX, YMIN, dY, ascale, hscale,
                            1.0 / dX, 1.0 / dY, 1.0 / ascale, 1.0 / hscale};
  h->tab_f = CylTab<float>{mmax, norder, numx, numy, cmap, (float)XMIN, (float)dX, (float)YMIN, (float)dY,
                           (float)ascale, (float)hscale, (float)(1.0 / dX), (float)(1.0 / dY),
                           (float)(1.0 / ascale), (float)(1.0 / hscale)};
  // FP32 copy of the tables for the separate mixed path, and the tiled
  // tables of the fused paths: FP32 roundings (the mixed path reads them
  // alone) and 16-bit remainders, which with them form the double-float
  // tables of the FP64 contraction and field (FP32-pipe arithmetic, 6 bytes
  // per entry against 8 for FP64).  A field block of the tiled layout reads
  // one contiguous region instead of hundreds of short row segments.
  h->pitch_f = (h->nnode + 3) & ~(size_t)3;
  const size_t rows = 8 * (size_t)(mmax + 1) * norder;
  const size_t nblk = (h->nnode + kTileNodes - 1) / kTileNodes;
  h->tile_rows = 6 * (size_t)(mmax + 1) * norder;
  const size_t ntile = nblk * h->tile_rows * kTileNodes;
  e = cudaMalloc((void**)&h->tab_f32, rows * h->pitch_f * sizeof(float) + ntile * (sizeof(float) + sizeof(short)));
  if (e == cudaSuccess) {
    h->tile_hi = h->tab_f32 + rows * h->pitch_f;
    h->tile_lo = reinterpret_cast<short*>(h->tile_hi + ntile);
    k_split_tab<<<grid_for((long long)(rows * h->pitch_f), 256, 8), 256>>>(h->tab, h->tab_f32, rows, h->nnode,
                                                                           h->pitch_f);
    k_tile_tab<<<grid_for((long long)ntile, 256, 8), 256>>>(h->tab, h->tile_hi, h->tile_lo, (mmax + 1) * norder,
                                                            h->nnode, nblk, TileOrder{numx + 1, numy + 1});
    e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    cudaFree(h->tab);
    if (h->tab_f32) cudaFree(h->tab_f32);
    delete h;
    return cuda_fail(e, "FP32 and tiled copies of the EOF tables");
  }
  *handle = h;
  return XT_OK;
}

int xt_cyl_table_destroy(void* handle) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  if (h) {
    h->fused.clear();
    if (h->capture) cudaStreamDestroy(h->capture);
    if (h->copy) cudaStreamDestroy(h->copy);
    for (cudaEvent_t& ev : h->qev)
      if (ev) cudaEventDestroy(ev);
    if (h->qdone) cudaEventDestroy(h->qdone);
    if (h->tab) cudaFree(h->tab);
    if (h->tab_f32) cudaFree(h->tab_f32);
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
  if (precision == XT_F64)
    k_cyl_contract_partial<double><<<g, 256, 0, st>>>(tab_ptr(h, 0), tab_ptr(h, 4), D, h->mmax, h->norder, h->nnode,
                                                      h->nnode, kContractChunks, part);
  else
    k_cyl_contract_partial<float><<<g, 256, 0, st>>>(tab_ptr_f32(h, 0), tab_ptr_f32(h, 4), D, h->mmax, h->norder,
                                                     h->nnode, h->pitch_f, kContractChunks, part);
  XT_CHECK_LAUNCH("k_cyl_contract_partial");
  k_cyl_contract_final<<<(nout + 127) / 128, 128, 0, st>>>(part, nout, kContractChunks, cos_out, sin_out, 0);
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
    if (sm > 48 * 1024) XT_CUDA(cudaFuncSetAttribute(k_cyl_field<double, TN, double>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_cyl_field<double, TN, double><<<blocks, 256, sm, st>>>(h->tab, cos_c, sin_c, h->mmax, h->norder, h->nnode,
                                                             h->nnode, mmax_use, nmax_use, nf,
                                                             static_cast<double*>(field));
  } else {
    const size_t sm = TN * mf * sizeof(float);
    if (sm > 48 * 1024) XT_CUDA(cudaFuncSetAttribute(k_cyl_field<float, TN, float>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_cyl_field<float, TN, float><<<blocks, 256, sm, st>>>(h->tab_f32, cos_c, sin_c, h->mmax, h->norder, h->nnode,
                                                           h->pitch_f, mmax_use, nmax_use, nf,
                                                           static_cast<float*>(field));
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


static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }


// Optional stage timing of xt_cyl_accumulate_eval: CUDA events recorded on the
// call's stream between its stages (binrec, scan, scatter, deposit, contract,
// field, eval), read back by xt_timing_read.  Off unless xt_timing_enable(1).
static thread_local int g_timing = 0;
static thread_local cudaEvent_t g_ev[8] = {};
static thread_local int g_nev = 0;

static int timing_mark(int k, cudaStream_t st) {
  if (!g_timing) return XT_OK;
  if (!g_ev[k]) XT_CUDA(cudaEventCreate(&g_ev[k]));
  XT_CUDA(cudaEventRecord(g_ev[k], st));
  g_nev = k + 1;
  return XT_OK;
}

struct FusedLayout {
  size_t grid, egrid, part, hist, flag, blist, off, tsum, rec, srec, field, stage, total;
  size_t hist_bytes;   // the bucket counts and the node-block flags after them, cleared together
};

// Particles in the first part of the sort when the results go to page-locked
// host memory (the parts are evaluated and copied out in turn); 0 for device
// results, which are sorted by cell alone, and for other host memory.
static int fused_qchunk(const CylHandle* h, long long n, bool staged) {
  const long long ncell = (long long)h->numx * h->numy;
  if (!staged || n <= 0 || kHostParts * ncell > (long long)kScanTile * kScanTile) return 0;
  return (int)std::max<long long>(32, ((3 * n + 7) / 8 + 31) & ~31LL);
}

// Parts of the host-result sort for part size qchunk (0: one part); the last
// part takes the rest of the particles.
static int host_parts(long long n, int qchunk) {
  return qchunk ? (int)std::min<long long>((n + qchunk - 1) / qchunk, kHostParts) : 1;
}

// From the pointer kinds of p0 p fr fp fz (kind[i] < 0: NULL): host_out,
// some of them are host memory; staged, all of those that are host memory are
// page-locked (their copies can run on a stream).
static void host_result_kinds(const int* kind, bool& host_out, bool& staged) {
  host_out = false;
  staged = true;
  for (int i = 0; i < 5; ++i) {
    if (kind[i] < 0) continue;
    host_out |= kind[i] != XT_PTR_DEVICE;
    staged &= kind[i] == XT_PTR_DEVICE || kind[i] == XT_PTR_PINNED;
  }
  staged &= host_out;
}

static FusedLayout fused_layout(const CylHandle* h, long long n, int precision) {
  const size_t rs = precision == XT_F32 ? sizeof(float) : sizeof(double);
  const size_t ncell = (size_t)h->numx * h->numy;
  FusedLayout L;
  size_t o = 0;
  auto take = [&](size_t b) { size_t at = o; o += align256(b); return at; };
  L.grid = take((size_t)(h->mmax + 1) * 2 * h->pitch_f * sizeof(double));   // planes of pitch_f nodes
  L.egrid = take((size_t)(h->mmax + 1) * 2 * h->pitch_f * sizeof(float));   // FP32 companion (error parts)
  L.part = take((size_t)(h->mmax + 1) * h->norder * 2 * kContractChunksDf * sizeof(double));
  const size_t nblk = (h->nnode + kTileNodes - 1) / kTileNodes;
  const size_t nbucket = kHostParts * ncell;   // (part, cell) buckets of the host-result sort
  L.hist_bytes = align256(nbucket * sizeof(int)) + nblk * sizeof(int);
  L.hist = take(L.hist_bytes);
  L.flag = L.hist + align256(nbucket * sizeof(int));
  L.blist = take((1 + nblk) * sizeof(int));
  L.off = take(nbucket * sizeof(int));
  L.tsum = take(kScanTile * sizeof(int));
  const size_t recb = precision == XT_F32 ? sizeof(BinRec<float>) : sizeof(BinRec<df>);
  L.rec = take((size_t)n * recb);
  L.srec = take((size_t)n * recb);
  L.field = take(h->nnode * (h->mmax + 1) * 6 * rs);
  L.stage = take((size_t)n * 5 * sizeof(double));   // p0 p fr fp fz of host-bound results
  L.total = o;
  return L;
}

int xt_cyl_field_engine(int engine) {
  XT_REQUIRE(engine >= 0 && engine <= 2, "field engine must be 0, 1 or 2, got %d", engine);
  g_field_engine = engine;
  return XT_OK;
}

int xt_cyl_active_blocks(void* handle, const void* workspace, long long n, int precision, int* active,
                         int* total) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  XT_REQUIRE(h && workspace && active && total, "NULL argument");
  XT_REQUIRE(n >= 0, "particle count must be >= 0");
  const FusedLayout L = fused_layout(h, n, precision);
  XT_CUDA(cudaDeviceSynchronize());
  XT_CUDA(cudaMemcpy(active, static_cast<const char*>(workspace) + L.blist, sizeof(int), cudaMemcpyDeviceToHost));
  *total = (int)((h->nnode + kTileNodes - 1) / kTileNodes);
  return XT_OK;
}

int xt_df_eval(int fn, const double* in, double* out, long long n, void* stream) {
  XT_REQUIRE(fn >= 0 && fn <= 2, "function must be 0, 1 or 2, got %d", fn);
  XT_REQUIRE(n >= 0 && (n == 0 || (in && out)), "bad arrays");
  if (int rc = upload_log_table()) return rc;
  if (n == 0) return XT_OK;
  cudaStream_t st = as_stream(stream);
  k_df_eval<<<resident_grid(k_df_eval, 256, 0, n), 256, 0, st>>>(fn, in, out, n);
  XT_CHECK_LAUNCH("k_df_eval");
  return XT_OK;
}

int xt_cyl_status(void) {
  int* err = nullptr;
  XT_CUDA(cudaDeviceSynchronize());
  XT_CUDA(cudaGetSymbolAddress((void**)&err, g_cyl_err));
  int v = 0;
  XT_CUDA(cudaMemcpy(&v, err, sizeof(int), cudaMemcpyDeviceToHost));
  if (v) {
    const int zero = 0;
    XT_CUDA(cudaMemcpy(err, &zero, sizeof(int), cudaMemcpyHostToDevice));
    set_error("cylindrical field: a bulk-copy wait timed out");
    return XT_ERR_DEVICE;
  }
  return XT_OK;
}

int xt_timing_enable(int on) {
  g_timing = on ? 1 : 0;
  g_nev = 0;
  return XT_OK;
}

int xt_timing_read(double* ms_out, int max) {
  XT_REQUIRE(ms_out && max >= 0, "NULL output");
  int k = 0;
  if (g_nev >= 2) {
    XT_CUDA(cudaEventSynchronize(g_ev[g_nev - 1]));
    for (; k < g_nev - 1 && k < max; ++k) {
      float ms = 0.f;
      XT_CUDA(cudaEventElapsedTime(&ms, g_ev[k], g_ev[k + 1]));
      ms_out[k] = ms;
    }
  }
  return k;
}

}  // extern "C"

// Arguments of the binning kernels, rebuilt to patch the captured node.
struct BinrecArgs {
  CylTab<double> Td;
  CylTab<float> Tf;
  BinrecDf K;
  const double *x, *y, *z, *m;
  long long n;
  int* hist;
  void* rec;
  double* rout;
  int nan;
  double* zd;
  float* ze;
  long long nz;
  int qchunk;
  void* p[15];
  void** list(bool f64) {
    int i = 0;
    if (f64) {
      p[i++] = &Td;
      p[i++] = &K;
    } else {
      p[i++] = &Tf;
    }
    for (void* a : {(void*)&x, (void*)&y, (void*)&z, (void*)&m, (void*)&n, (void*)&hist, (void*)&rec, (void*)&rout,
                    (void*)&nan, (void*)&zd, (void*)&ze, (void*)&nz, (void*)&qchunk})
      p[i++] = a;
    return p;
  }
};

static BinrecDf binrec_constants(const CylTab<double>& T) {
  return BinrecDf{host_df(T.XMIN), host_df(T.inv_dX), host_df(T.YMIN), host_df(T.inv_dY), host_df(T.inv_ascale),
                  host_df(T.inv_hscale), host_df(1.0e-10), host_df(1.0e-8), host_df(-FOUR_PI_C)};
}

// Copies of staged results (qchunk > 0) to outs[0..4], part q on the copy
// stream behind the event the evaluation of that part recorded; the stream
// st then waits for all of them.  Called right after the enqueue, under
// copy_mu, so that the events are this call's.
static int stage_copies(CylHandle* h, const FusedLayout& L, void* workspace, long long n, int qchunk,
                        double* const* outs, cudaStream_t st) {
  const double* stage = reinterpret_cast<const double*>(static_cast<char*>(workspace) + L.stage);
  const int npart = host_parts(n, qchunk);
  // the five results as consecutive arrays of n (the stage's own layout): one
  // 2D copy per part instead of five
  // (pitches up to 2^31 - 1 bytes, the copy API's limit)
  bool block = outs[0] != nullptr && (size_t)n * sizeof(double) <= (size_t)INT_MAX;
  for (int k = 1; k < 5 && block; ++k) block = outs[k] == outs[0] + (size_t)k * n;
  for (int q = 0; q < npart; ++q) {
    XT_CUDA(cudaStreamWaitEvent(h->copy, h->qev[q], 0));
    const long long p0 = (long long)q * qchunk, np = q + 1 < npart ? qchunk : n - p0;
    if (block) {
      XT_CUDA(cudaMemcpy2DAsync(outs[0] + p0, (size_t)n * sizeof(double), stage + p0, (size_t)n * sizeof(double),
                                (size_t)np * sizeof(double), 5, cudaMemcpyDefault, h->copy));
      continue;
    }
    for (int k = 0; k < 5; ++k)
      if (outs[k])
        XT_CUDA(cudaMemcpyAsync(outs[k] + p0, stage + (size_t)k * n + p0, (size_t)np * sizeof(double),
                                cudaMemcpyDefault, h->copy));
  }
  XT_CUDA(cudaEventRecord(h->qdone, h->copy));
  XT_CUDA(cudaStreamWaitEvent(st, h->qdone, 0));
  return XT_OK;
}

// Launch the fused call as a CUDA graph.  A call whose shape, workspace and
// result arrays match the cached graph's replays it, with the binning node
// pointed at this call's particle arrays and R; the second consecutive call of
// a new shape captures it (on the handle's private stream); any other call is
// enqueued directly.  One graph launch replaces two memsets and nine kernel
// launches.  If capture fails, the call is enqueued directly.
template <typename Enq>
static int fused_graph_launch(CylHandle* h, int precision, const double* x, const double* y, const double* z,
                              const double* m, long long n, int m1, int m2, int nan_to_origin, double* cos_out,
                              double* sin_out, double* const* outs, void* workspace, const FusedLayout& L,
                              int qchunk, cudaStream_t& st, Enq&& enqueue) {
  std::lock_guard<std::mutex> lock(h->graph_mu);
  FusedGraph& G = h->fused;
  FusedGraph::Key key{n, precision, m1, m2, nan_to_origin, workspace, cos_out, sin_out,
                      {outs[0], outs[1], outs[2], outs[3], outs[4]}, g_field_engine, qchunk};
  const bool f64 = precision == XT_F64;
  if (!G.valid || !G.key.same(key)) {
    if (!(G.seen && G.last.same(key))) {     // first sighting of this shape: run it directly
      G.seen = true;
      G.last = key;
      return enqueue();
    }
    G.clear();
    if (!h->capture) XT_CUDA(cudaStreamCreateWithFlags(&h->capture, cudaStreamNonBlocking));
    const cudaStream_t user = st;
    st = h->capture;
    XT_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue();
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    st = user;
    if (rc != XT_OK || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      G.seen = false;
      return enqueue();
    }
    G.graph = g;
    size_t nn = 0;
    XT_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    XT_CUDA(cudaGraphGetNodes(g, nodes.data(), &nn));
    const void* want = f64 ? (const void*)k_cyl_binrec_df : (const void*)k_cyl_binrec<float>;
    for (cudaGraphNode_t nd : nodes) {
      cudaGraphNodeType t;
      XT_CUDA(cudaGraphNodeGetType(nd, &t));
      if (t != cudaGraphNodeTypeKernel) continue;
      cudaKernelNodeParams kp{};
      XT_CUDA(cudaGraphKernelNodeGetParams(nd, &kp));
      if (kp.func == want) {
        G.binrec = nd;
        G.bp = kp;
      }
    }
    const cudaError_t ei = G.binrec ? cudaGraphInstantiate(&G.exec, g, 0) : cudaErrorInvalidValue;
    if (ei != cudaSuccess) {
      // no patchable binning node, or no executable graph: run this call (and
      // the next of this shape) directly, as after a failed capture
      G.clear();
      cudaGetLastError();
      G.seen = false;
      return enqueue();
    }
    G.key = key;
    G.x = x;
    G.y = y;
    G.z = z;
    G.m = m;
    G.rout = outs[5];
    G.valid = true;
  } else if (G.x != x || G.y != y || G.z != z || G.m != m || G.rout != outs[5]) {
    char* ws = static_cast<char*>(workspace);
    BinrecArgs a{h->tab_d, h->tab_f, binrec_constants(h->tab_d), x, y, z, m, n,
                 reinterpret_cast<int*>(ws + L.hist), ws + L.rec, outs[5], nan_to_origin,
                 reinterpret_cast<double*>(ws + L.grid), reinterpret_cast<float*>(ws + L.egrid),
                 (long long)(h->mmax + 1) * 2 * (long long)h->pitch_f, qchunk, {}};
    cudaKernelNodeParams kp = G.bp;
    kp.kernelParams = a.list(f64);
    kp.extra = nullptr;
    XT_CUDA(cudaGraphExecKernelNodeSetParams(G.exec, G.binrec, &kp));
    G.x = x;
    G.y = y;
    G.z = z;
    G.m = m;
    G.rout = outs[5];
  }
  XT_CUDA(cudaGraphLaunch(G.exec, st));
  return XT_OK;
}

extern "C" {

size_t xt_cyl_accumulate_eval_workspace(void* handle, long long n, int precision) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  if (!h || n < 0) return 0;
  return fused_layout(h, n, precision).total;
}

}  // extern "C"

// The stages of the sorted pipeline on one snapshot: binning (per-particle
// set-up once, records with the particle's cell), counting sort by cell (by
// part of the particle range, then cell, when results go to host memory),
// then with do_acc the run-accumulated deposit and the contraction into
// cos_out/sin_out, and with do_eval the field from cos_src/sin_src and the
// evaluation into outs (p0 p fr fp fz; R, outs[5], is written by the binning
// kernel when non-NULL).  Host results (host_out) are staged and copied out a
// part at a time behind the evaluation.
static int sorted_enqueue(CylHandle* h, const FusedLayout& L, void* workspace, const double* x, const double* y,
                          const double* z, const double* m, long long n, int precision, int m1, int m2,
                          int nan_to_origin, bool do_acc, bool do_eval, double* cos_out, double* sin_out,
                          const double* cos_src, const double* sin_src, double* const* outs, bool host_out,
                          int qchunk, cudaStream_t st) {
  char* ws = static_cast<char*>(workspace);
  double* D = reinterpret_cast<double*>(ws + L.grid);
  float* E = reinterpret_cast<float*>(ws + L.egrid);
  double* part = reinterpret_cast<double*>(ws + L.part);
  int* hist = reinterpret_cast<int*>(ws + L.hist);
  int* off = reinterpret_cast<int*>(ws + L.off);
  int* tsum = reinterpret_cast<int*>(ws + L.tsum);
  const int ncell = h->numx * h->numy;
  const int nblk = (int)((h->nnode + kTileNodes - 1) / kTileNodes);
  // results bound for host memory: records sorted by (part, cell), the parts
  // evaluated in turn and copied out behind the evaluation
  const int npart = host_parts(n, qchunk);
  const int nbucket = qchunk ? npart * ncell : ncell;
  ActiveBlocks ab;
  ab.flag = reinterpret_cast<int*>(ws + L.flag);
  ab.list = reinterpret_cast<int*>(ws + L.blist);
  ab.numy = h->numy;
  ab.ncell = ncell;
  ab.nblk = nblk;
  ab.to = TileOrder{h->numx + 1, h->numy + 1};
  const long long ngrid = (long long)(h->mmax + 1) * 2 * (long long)h->pitch_f;   // entries of D and of E
  auto run = [&](auto tag) -> int {
    // the binning kernel zeroes D and E; without particles they are cleared here
    if (n == 0 && do_acc) {
      XT_CUDA(cudaMemsetAsync(D, 0, (size_t)ngrid * sizeof(double), st));
      XT_CUDA(cudaMemsetAsync(E, 0, (size_t)ngrid * sizeof(float), st));
    }
    XT_CUDA(cudaMemsetAsync(hist, 0, L.hist_bytes, st));   // cell counts and node-block flags
    // without particles no node block is read (the scans that list them do not run)
    if (n == 0) XT_CUDA(cudaMemsetAsync(ab.list, 0, sizeof(int), st));
    using R = decltype(tag);
    constexpr bool F64 = std::is_same<R, double>::value;
    using RT = typename std::conditional<F64, df, float>::type;   // record arithmetic
    const CylTab<R>& T = *reinterpret_cast<const CylTab<R>*>(F64 ? (const void*)&h->tab_d : (const void*)&h->tab_f);
    BinRec<RT>* rec = reinterpret_cast<BinRec<RT>*>(ws + L.rec);
    BinRec<RT>* srec = reinterpret_cast<BinRec<RT>*>(ws + L.srec);
    R* field = reinterpret_cast<R*>(ws + L.field);
    int rc;
    if ((rc = timing_mark(0, st))) return rc;
    if (n > 0) {
      if constexpr (F64) {
        const BinrecDf K = binrec_constants(T);
        k_cyl_binrec_df<<<resident_grid(k_cyl_binrec_df, 256, 0, n), 256, 0, st>>>(
            T, K, x, y, z, m, n, hist, rec, outs[5], nan_to_origin, D, E, ngrid, qchunk);
      } else {
        k_cyl_binrec<float><<<resident_grid(k_cyl_binrec<float>, 256, 0, n), 256, 0, st>>>(
            T, x, y, z, m, n, hist, rec, outs[5], nan_to_origin, D, E, ngrid, qchunk);
      }
      XT_CHECK_LAUNCH("k_cyl_binrec");
      if ((rc = timing_mark(1, st))) return rc;
      {
        const int ntile = (nbucket + kScanTile - 1) / kScanTile;
        k_scan_tiles<<<ntile, kScanTile, 0, st>>>(hist, off, tsum, nbucket, ab);
        XT_CHECK_LAUNCH("k_scan_tiles");
        k_scan_add<<<ntile, kScanTile, 0, st>>>(off, tsum, nbucket, ntile, ab);
        XT_CHECK_LAUNCH("k_scan_add");
      }
      if ((rc = timing_mark(2, st))) return rc;
      k_cyl_scatter<RT><<<resident_grid(k_cyl_scatter<RT>, 256, 0, n), 256, 0, st>>>(n, off, rec, srec, qchunk,
                                                                                      ncell);
      XT_CHECK_LAUNCH("k_cyl_scatter");
      if ((rc = timing_mark(3, st))) return rc;
      if (do_acc) {
      // Run length: particles summed in registers per lane before the atomics.
      // Measured on 1e6 disc particles with same-cell lanes merged before the
      // atomics (runs of 4 to 16): 4 in both precisions (FP64 deposit 0.096 ms
      // against 0.100 at 8 and 0.126 at 16), one block per 128 runs (the
      // hardware fills later waves as blocks end).
      auto dep = [&](auto mc) {
        constexpr int MC = decltype(mc)::value;
        using Mth = std::conditional_t<F64, DepDF, DepF32>;
        constexpr int NP = F64 ? 2 : 1;
        // (one pass with 2-3 blocks per SM, or two passes with 2-3, measured
        // 0.127-0.131 ms against 0.121 ms for two passes at 4 blocks per SM)
        auto kern = k_cyl_deposit_sorted<Mth, MC, NP>;
        const int run = 4;
        const long long nrun = (n + run - 1) / run;
        const int grid = (int)std::min<long long>((nrun + 127) / 128, 8LL * resident_grid(kern, 128, 0, nrun));
        kern<<<grid, 128, 0, st>>>(h->numy, h->numx + 1, h->mmax, n, run, srec, D, E, h->pitch_f);
      };
      if (h->mmax <= 2) dep(std::integral_constant<int, 2>{});
      else if (h->mmax <= 4) dep(std::integral_constant<int, 4>{});
      else if (h->mmax <= 6) dep(std::integral_constant<int, 6>{});
      else dep(std::integral_constant<int, 8>{});
      XT_CHECK_LAUNCH("k_cyl_deposit_sorted");
      }
    } else {
      for (int k = 1; k <= 3; ++k)
        if ((rc = timing_mark(k, st))) return rc;
    }
    if ((rc = timing_mark(4, st))) return rc;
    if (do_acc) {
    // coefficient contraction in both precisions from the double-float tables:
    // order groups of kContractRows, node chunks sized for one wave
    // (3 and 6 orders per block measured alike, 9 slower: fewer resident blocks)
    const int ngroup = (h->norder + kContractRows - 1) / kContractRows;
    const int npair = 2 * h->mmax + 1;
    const int cap = resident_blocks_per_sm((const void*)k_cyl_contract_df<kContractRows>, 128, 0) * sm_count();
    const int nch = std::max(1, std::min(kContractChunksDf, cap / (ngroup * npair)));
    k_cyl_contract_df<kContractRows><<<dim3(nch * ngroup, npair), 128, 0, st>>>(
        h->tile_hi, h->tile_lo, h->pitch_f, D, E, h->mmax, h->norder, h->nnode, nch, ngroup, ab.list, part);
    XT_CHECK_LAUNCH("k_cyl_contract_df");
    // (the sum of the partials folded into the contraction's last block was
    // measured no faster)
    const int nout = (h->mmax + 1) * h->norder * 2;
    k_cyl_contract_final<<<(nout + 127) / 128, 128, 0, st>>>(part, nout, nch, cos_out, sin_out, h->norder);
    XT_CHECK_LAUNCH("k_cyl_contract_final");
    }
    if ((rc = timing_mark(5, st))) return rc;
    if (!do_eval) return timing_mark(6, st);
    // FP64 path: double-float field from the double-float tables; mixed path:
    // FP32 field from the FP32 tables (coefficients staged as df in both)
    using FT = std::conditional_t<F64, df, float>;
    FieldBulkPlan P;
    const bool bulk = g_field_engine != 2 && field_bulk_plan(h, F64, P);
    XT_REQUIRE(bulk || g_field_engine != 1, "the bulk-copy field pipeline does not fit M = %d, Q = %d", h->mmax,
               h->norder);
    if (bulk) {
      // bulk-copy pipeline: one persistent CTA per SM over the node blocks
      auto kern = k_cyl_field_bulk<FT, F64>;
      XT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.smem));
      static int* err = nullptr;
      if (!err) XT_CUDA(cudaGetSymbolAddress((void**)&err, g_cyl_err));
      const int grid = std::min(nblk, sm_count());
      kern<<<grid, kFieldThreads, P.smem, st>>>(h->tile_hi, h->tile_lo, cos_src, sin_src, h->mmax, h->norder,
                                                h->nnode, ab.to, ab.list, P.mg, P.nstage, P.stage_hi, P.stage, P.cf,
                                                reinterpret_cast<FT*>(field), err);
    } else {
      // row loads: one block per node block of the tiled tables, 224 threads
      // (the 672 (m, field, quad) tasks of a 64-node block in three rounds,
      // four blocks per SM), six rows in flight.  Measured on the 257^2-node,
      // M = 6, Q = 18 table: 0.059 ms against 0.067 (256 threads), 0.066 (672)
      // and 0.072 (96).
      constexpr int RB = 6, NT = 224, MINB = 4;
      const size_t sm = 2 * (size_t)(h->mmax + 1) * h->norder * sizeof(df) +
                        kTileNodes * (size_t)(h->mmax + 1) * 6 * sizeof(FT);
      if (sm > 48 * 1024)
        XT_CUDA(cudaFuncSetAttribute(k_cyl_field2<FT, F64, RB, NT, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sm));
      k_cyl_field2<FT, F64, RB, NT, MINB><<<nblk, NT, sm, st>>>(h->tile_hi, h->tile_lo, cos_src, sin_src, h->mmax,
                                                                h->norder, h->nnode, ab.to, ab.list,
                                                                reinterpret_cast<FT*>(field));
    }
    XT_CHECK_LAUNCH(bulk ? "k_cyl_field_bulk" : "k_cyl_field2");
    if ((rc = timing_mark(6, st))) return rc;
    if (n > 0) {
      // The evaluation runs over the sorted records (neighbouring threads share
      // field rows in L1: 0.18 ms against 0.39 ms in particle order for 1e6
      // disc particles) and writes each result to its particle's slot.  Results
      // bound for host memory are staged in the workspace, one part of the
      // particles at a time (the records are sorted by part, then cell); a
      // part's five result blocks are copied out on the copy stream while the
      // next part is evaluated, so the host-link transfer overlaps all but one
      // part of the evaluation.
      // (Host results on a table too large for the part buckets are
      // evaluated in particle order instead, with coalesced writes over the
      // link.)
      auto eval = [&](double* const* o, const int* rb, const int* re, long long nmax, auto srt) {
        constexpr bool S = decltype(srt)::value;
        const BinRec<RT>* er = S ? srec : rec;
        if constexpr (F64) {
          auto kern = k_cyl_eval_sorted_df<S>;
          kern<<<resident_grid(kern, 128, 0, nmax), 128, 0, st>>>(T, reinterpret_cast<const df*>(field), n, er, m1,
                                                                 m2, o[0], o[1], o[2], o[3], o[4], rb, re);
        } else {
          CylEvalOpts eo;
          eo.mode = XT_CYL_ACCUMULATED_EVAL_PARTICLES; eo.m1 = m1; eo.m2 = m2; eo.mmax_use = h->mmax; eo.no_odd = 0;
          eo.perturb = 0; eo.density = 0; eo.nf = 6;
          auto kern = k_cyl_eval_sorted<R, S>;
          kern<<<resident_grid(kern, 128, 0, nmax), 128, 0, st>>>(T, field, n, er, eo, o[0], o[1], o[2], o[3], o[4],
                                                                  rb, re);
        }
        XT_CHECK_LAUNCH("k_cyl_eval_sorted");
        return XT_OK;
      };
      if (!qchunk) {
        if (host_out) rc = eval(outs, nullptr, nullptr, n, std::false_type{});
        else rc = eval(outs, nullptr, nullptr, n, std::true_type{});
        if (rc) return rc;
      } else {
        // part q evaluated: event qev[q] (an external event node when the call
        // is being captured), behind which stage_copies copies it out
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        XT_CUDA(cudaStreamIsCapturing(st, &cs));
        const unsigned evf = cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
        double* stage = reinterpret_cast<double*>(ws + L.stage);
        double* so[5];
        for (int k = 0; k < 5; ++k) so[k] = outs[k] ? stage + (size_t)k * n : nullptr;
        for (int q = 0; q < npart; ++q) {
          const int* rb = off + (size_t)q * ncell;
          const int* re = q + 1 < npart ? off + (size_t)(q + 1) * ncell : nullptr;
          const long long np = q + 1 < npart ? qchunk : n - (long long)q * qchunk;
          if ((rc = eval(so, rb, re, np, std::true_type{}))) return rc;
          XT_CUDA(cudaEventRecordWithFlags(h->qev[q], st, evf));
        }
      }
    }
    return timing_mark(7, st);
  };
  return precision == XT_F64 ? run(double{}) : run(float{});
}

extern "C" {

int xt_cyl_accumulate_eval(void* handle, const double* x, const double* y, const double* z, const double* m,
                           long long n, int precision, int m1, int m2, int nan_to_origin, double* cos_out,
                           double* sin_out, double* const* outs, void* workspace, size_t workspace_bytes,
                           void* stream) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  XT_REQUIRE(h, "NULL table handle");
  XT_REQUIRE(n >= 0 && n < (1LL << 31), "particle count must be in [0, 2^31)");
  XT_REQUIRE(cos_out && sin_out && outs, "NULL output");
  XT_REQUIRE(n == 0 || (x && y && z && m), "NULL particle array");
  XT_REQUIRE(precision == XT_F64 || precision == XT_F32, "bad precision %d", precision);
  XT_REQUIRE(h->mmax <= 8 && h->norder <= 24, "the fused path supports mmax <= 8, norder <= 24 (got %d, %d)",
             h->mmax, h->norder);
  XT_REQUIRE((long long)h->numx * h->numy <= (long long)kScanTile * kScanTile,
             "the fused path supports numx*numy <= %d cells", kScanTile * kScanTile);
  // particle arrays and results may live in host memory the device can
  // address (pinned, or any host memory where the device has pageable access)
  bool host_out = false, staged = false;
  if (n > 0) {
    for (const void* p : {(const void*)x, (const void*)y, (const void*)z, (const void*)m})
      XT_REQUIRE(pointer_access(p) != XT_PTR_INACCESSIBLE, "particle array %p is host memory the device cannot address",
                 p);
    int kind[6];
    for (int i = 0; i < 6; ++i) {
      kind[i] = outs[i] ? pointer_access(outs[i]) : -1;
      XT_REQUIRE(kind[i] != XT_PTR_INACCESSIBLE, "result array %d is host memory the device cannot address", i);
    }
    // R (outs[5]) is written coalesced by the binning kernel
    host_result_kinds(kind, host_out, staged);
  }
  const int qchunk = fused_qchunk(h, n, staged);
  const FusedLayout L = fused_layout(h, n, precision);
  if (!workspace || workspace_bytes < L.total) {
    set_error("workspace of %zu bytes needed, %zu given", L.total, workspace_bytes);
    return XT_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);   // the stream work is enqueued on (the capture stream while capturing)
  auto enqueue = [&]() -> int {
    return sorted_enqueue(h, L, workspace, x, y, z, m, n, precision, m1, m2, nan_to_origin, true, true, cos_out,
                          sin_out, cos_out, sin_out, outs, host_out, qchunk, st);
  };
  std::unique_lock<std::mutex> lock(h->copy_mu, std::defer_lock);
  if (qchunk) lock.lock();
  int rc;
  // Stage timing records events between the launches: enqueue directly.
  if (g_timing || n == 0) rc = enqueue();
  else
    rc = fused_graph_launch(h, precision, x, y, z, m, n, m1, m2, nan_to_origin, cos_out, sin_out, outs, workspace,
                            L, qchunk, st, enqueue);
  if (rc || !qchunk) return rc;
  return stage_copies(h, L, workspace, n, qchunk, outs, st);
}


// Shared argument checks of the sorted entry points; sets host_out and staged
// as host_result_kinds does.
static int sorted_checks(const CylHandle* h, const double* x, const double* y, const double* z, const double* m,
                         long long n, int precision, double* const* outs, int nouts, bool& host_out, bool& staged) {
  XT_REQUIRE(h, "NULL table handle");
  XT_REQUIRE(n >= 0 && n < (1LL << 31), "particle count must be in [0, 2^31)");
  XT_REQUIRE(n == 0 || (x && y && z && m), "NULL particle array");
  XT_REQUIRE(precision == XT_F64 || precision == XT_F32, "bad precision %d", precision);
  XT_REQUIRE(h->mmax <= 8 && h->norder <= 24, "the sorted path supports mmax <= 8, norder <= 24 (got %d, %d)",
             h->mmax, h->norder);
  XT_REQUIRE((long long)h->numx * h->numy <= (long long)kScanTile * kScanTile,
             "the sorted path supports numx*numy <= %d cells", kScanTile * kScanTile);
  host_out = staged = false;
  if (n > 0) {
    for (const void* p : {(const void*)x, (const void*)y, (const void*)z, (const void*)m})
      XT_REQUIRE(pointer_access(p) != XT_PTR_INACCESSIBLE, "particle array %p is host memory the device cannot address",
                 p);
    int kind[6] = {-1, -1, -1, -1, -1, -1};
    for (int i = 0; i < nouts && i < 6; ++i) {
      kind[i] = outs[i] ? pointer_access(outs[i]) : -1;
      XT_REQUIRE(kind[i] != XT_PTR_INACCESSIBLE, "result array %d is host memory the device cannot address", i);
    }
    host_result_kinds(kind, host_out, staged);
  }
  return XT_OK;
}

int xt_cyl_accumulate_sorted(void* handle, const double* x, const double* y, const double* z, const double* m,
                             long long n, int precision, int nan_to_origin, double* cos_out, double* sin_out,
                             void* workspace, size_t workspace_bytes, void* stream) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  bool host_out = false, staged = false;
  double* const none[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  int rc = sorted_checks(h, x, y, z, m, n, precision, none, 6, host_out, staged);
  if (rc) return rc;
  XT_REQUIRE(cos_out && sin_out, "NULL output");
  XT_REQUIRE(pointer_access(cos_out) != XT_PTR_INACCESSIBLE && pointer_access(sin_out) != XT_PTR_INACCESSIBLE,
             "coefficient output is host memory the device cannot address");
  const FusedLayout L = fused_layout(h, n, precision);
  if (!workspace || workspace_bytes < L.total) {
    set_error("workspace of %zu bytes needed, %zu given", L.total, workspace_bytes);
    return XT_ERR_WORKSPACE;
  }
  return sorted_enqueue(h, L, workspace, x, y, z, m, n, precision, 0, 0, nan_to_origin, true, false, cos_out,
                        sin_out, nullptr, nullptr, none, false, 0, as_stream(stream));
}

int xt_cyl_eval_sorted(void* handle, const double* x, const double* y, const double* z, long long n, int precision,
                       int m1, int m2, const double* cos_c, const double* sin_c, double* const* outs,
                       void* workspace, size_t workspace_bytes, void* stream) {
  CylHandle* h = static_cast<CylHandle*>(handle);
  XT_REQUIRE(outs, "NULL output list");
  bool host_out = false, staged = false;
  // the binning kernel reads a mass per particle for the deposit weight, which
  // evaluation does not use: it is given the x array
  int rc = sorted_checks(h, x, y, z, x, n, precision, outs, 6, host_out, staged);
  if (rc) return rc;
  XT_REQUIRE(cos_c && sin_c, "NULL coefficients");
  XT_REQUIRE(pointer_access(cos_c) != XT_PTR_INACCESSIBLE && pointer_access(sin_c) != XT_PTR_INACCESSIBLE,
             "coefficients are host memory the device cannot address");
  const FusedLayout L = fused_layout(h, n, precision);
  if (!workspace || workspace_bytes < L.total) {
    set_error("workspace of %zu bytes needed, %zu given", L.total, workspace_bytes);
    return XT_ERR_WORKSPACE;
  }
  const int qchunk = fused_qchunk(h, n, staged);
  std::unique_lock<std::mutex> lock(h->copy_mu, std::defer_lock);
  if (qchunk) lock.lock();
  rc = sorted_enqueue(h, L, workspace, x, y, z, x, n, precision, m1, m2, 0, false, true, nullptr, nullptr, cos_c,
                      sin_c, outs, host_out, qchunk, as_stream(stream));
  if (rc || !qchunk) return rc;
  return stage_copies(h, L, workspace, n, qchunk, outs, as_stream(stream));
}

}  // extern "C"
