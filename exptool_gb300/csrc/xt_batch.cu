// Batched spherical accumulation over many snapshots in one persistent launch.
//
// Workload: spheresl.compute_coefficients (spheresl.py:439-475) applied to a
// time series of snapshots, the reference's natural caller for coefficient
// series.  Particles of all snapshots are one FP32 xyzm stream (float4 per
// particle); snapshot s owns particles [offsets[s], offsets[s+1]).
//
// Each particle's contribution -4 pi m Y_lm(theta, phi) plerp x {x1, x2} goes
// to the two radial nodes it interpolates between (the reorganisation of the
// single-snapshot FP64 kernel, xt_sph.cu).  Here the node grid of a block of
// coefficient rows lives in shared memory: a CTA takes a work item (snapshot,
// particle chunk, row part) from a global counter, deposits the chunk with
// FP32 shared-memory atomics, then adds its grid into the snapshot's FP64 grid
// in global memory (FP64 atomics, one per non-zero node value).  A batched
// FP64 kernel contracts every snapshot grid with the radial tables.  No CTA
// ever waits on another; the loop ends when the counter passes the last item.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>

#include "xt_internal.cuh"
#include "xt_launch.cuh"
#include "xt_df.cuh"

namespace xt {

struct BatchItem {
  int snap;
  int part;           // radial node part
  long long begin, end;
};

constexpr float FOUR_PI_F = 12.566370614359172f;

// Work items split the radial nodes: part k owns particles whose lower
// interpolation node i lies in [ilo_k, ihi_k) and keeps a shared grid of all
// rows over nodes [ilo_k, ihi_k] (node ihi_k is shared with the next part;
// both parts add their share of it to the FP64 grid).  Particles outside the
// part's range are skipped after the radial mapping, so Legendre functions,
// trigonometry and deposits are computed once per particle.
template <int LCAP>
__global__ void k_sph_batched(SphTab<float> T, const float4* __restrict__ xyzm, const BatchItem* __restrict__ items,
                              int nitems, int* __restrict__ counter, const int* __restrict__ part_nodes, int no_odd,
                              double* __restrict__ G) {
  extern __shared__ float sg[];
  __shared__ int s_item;
  constexpr int NT = (LCAP + 1) * (LCAP + 2) / 2;
  const int numr = T.numr;
  const int nrow = (T.lmax + 1) * (T.lmax + 1);
  const int lstride = T.lmax + 1;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) break;
    const BatchItem I = items[it];
    const int ilo = part_nodes[I.part], ihi = part_nodes[I.part + 1];
    const int span = ihi - ilo + 1;               // nodes ilo..ihi
    const int ncell = nrow * span;
    for (int k = threadIdx.x; k < ncell; k += blockDim.x) sg[k] = 0.f;
    __syncthreads();
    long long p = I.begin + threadIdx.x;
    float4 q = (p < I.end) ? xyzm[p] : make_float4(0.f, 0.f, 0.f, 0.f);
    for (; p < I.end; p += blockDim.x) {
      const long long pn = p + blockDim.x;
      const float4 qn = (pn < I.end) ? xyzm[pn] : q;    // next particle in flight
      float r = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z);
      if (!(r >= 1.0e-10f)) r = 1.0e-10f;
      const SphBins<float> B = sph_bins(T, r, false, false);
      if (B.i >= ilo && B.i < ihi) {
        const float costh = q.z / r;
        float c1, s1;
        unit_phi(q.x, q.y, c1, s1);
        float P[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) P[k] = 0.f;
        legendre<float, LCAP>(costh, T.lmax, P);
        float cm[LCAP + 1], sm[LCAP + 1];
        multiples<float, LCAP>(c1, s1, T.lmax, cm, sm);
        const float base = -FOUR_PI_F * q.w;
        const float w0 = B.lw0 * base, w1 = B.lw1 * base;
        float* g0 = sg + (B.i - ilo);
#pragma unroll
        for (int l = 0; l <= LCAP; ++l) {
          if (l > T.lmax) break;
          if (no_odd && (l & 1)) continue;
          const int loff = l * l;
#pragma unroll
          for (int m = 0; m <= l; ++m) {
            const float a = T.fact[l * lstride + m] * P[tri(l, m)];
            const int rc = (m == 0) ? loff : loff + 2 * m - 1;
            const float v = (m == 0) ? a : a * cm[m];
            atomicAdd(g0 + rc * span, v * w0);
            atomicAdd(g0 + rc * span + 1, v * w1);
            if (m > 0) {
              const float u = a * sm[m];
              atomicAdd(g0 + (rc + 1) * span, u * w0);
              atomicAdd(g0 + (rc + 1) * span + 1, u * w1);
            }
          }
        }
      }
      q = qn;
    }
    __syncthreads();
    double* gs = G + (size_t)I.snap * nrow * numr + ilo;
    for (int k = threadIdx.x; k < ncell; k += blockDim.x) {
      const float v = sg[k];
      if (v != 0.f) {
        const int row = k / span, node = k - row * span;
        atomicAdd(gs + (size_t)row * numr + node, (double)v);
      }
    }
    __syncthreads();
  }
}

// expcoef[s, row, n] = sum_node efp[l, n, node] G[s, row, node] in double-float
// arithmetic on the FP32 pipe (the FP64 pipe of GB300 issues at a small
// fraction of the FP32 rate).  One block per (snapshot, l): tiles of 128
// nodes of the 2l+1 grid rows (split into FP32 pairs on loading) and of the
// split table rows of this l are staged in shared memory.  The (2l+1) nmax
// outputs share the 256 threads evenly: each output's nodes are split over
// S = 256 / outputs slices (node j to slice j mod S), each slice keeping a
// lazily renormalised df sum, and the slices are merged in shared memory at
// the end (for 2l+1 = 13, nmax = 20, S = 1 and four threads take a second
// output).  Error ~numr 2^-47 of the sum of |terms|.
constexpr int kCbTile = 128;
constexpr int kCbPitch = kCbTile + 1;      // float2 pitch: rows of the table tile fall in distinct banks
constexpr int kCbOut = 3;                  // outputs per thread when S = 1: (2l+1) nmax <= 3 * 256
constexpr int kCbThreads = 256;

__device__ __forceinline__ float2 cb_pair(double v) {
  const df d = df_from(v);
  return make_float2(d.h, d.l);
}
__device__ __forceinline__ float2 cb_pair(float2 v) { return v; }

template <typename GT>
__global__ void __launch_bounds__(kCbThreads) k_sph_contract_batched_df(const float2* __restrict__ efp_df,
                                                                       const GT* __restrict__ G, int lmax,
                                                                       int nmax, int numr,
                                                                       double* __restrict__ out) {
  extern __shared__ float2 cb_sm[];
  __shared__ float2 red[kCbThreads];
  const int s = blockIdx.x, l = blockIdx.y;
  const int nrow = (lmax + 1) * (lmax + 1), r0 = l * l, nr = 2 * l + 1;
  const int nout = nr * nmax;
  const int S = nout >= kCbThreads ? 1 : kCbThreads / nout;    // node slices per output
  float2* Gt = cb_sm;                       // [nr][kCbPitch]
  float2* Et = cb_sm + nr * kCbPitch;       // [nmax][kCbPitch]
  const GT* g = G + ((size_t)s * nrow + r0) * numr;
  const float2* e = efp_df + (size_t)l * nmax * numr;
  const int tid = threadIdx.x;
  const int sl = tid % S, o0 = tid / S;     // slice and first output of this thread
  dacc acc[kCbOut];
  // outputs o0 + q * (256 / S), as (row offset, order offset) into the tiles
  int go[kCbOut], eo[kCbOut];
  int nq = 0;
#pragma unroll
  for (int q = 0; q < kCbOut; ++q) {
    const int o = o0 + q * (kCbThreads / S);
    const bool have = o < nout && (q == 0 || S == 1);
    const int r = have ? o / nmax : 0, n = have ? o - r * nmax : 0;
    go[q] = r * kCbPitch;
    eo[q] = n * kCbPitch;
    if (have) nq = q + 1;
  }
  for (int t0 = 0; t0 < numr; t0 += kCbTile) {
    const int tn = min(kCbTile, numr - t0);
    __syncthreads();
    for (int k = tid; k < nr * kCbTile; k += kCbThreads) {
      const int r = k / kCbTile, j = k - r * kCbTile;
      Gt[r * kCbPitch + j] = j < tn ? cb_pair(g[(size_t)r * numr + t0 + j]) : make_float2(0.f, 0.f);
    }
    for (int k = tid; k < nmax * kCbTile; k += kCbThreads) {
      const int n = k / kCbTile, j = k - n * kCbTile;
      Et[n * kCbPitch + j] = j < tn ? e[(size_t)n * numr + t0 + j] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    if (nq == 1) {
#pragma unroll 4
      for (int j = sl; j < tn; j += S) {
        const float2 a = Gt[go[0] + j], b = Et[eo[0] + j];
        acc[0].fma(df{a.x, a.y}, df{b.x, b.y});
      }
    } else if (nq > 1) {
      for (int j = 0; j < tn; ++j) {
#pragma unroll
        for (int q = 0; q < kCbOut; ++q) {
          if (q < nq) {
            const float2 a = Gt[go[q] + j], b = Et[eo[q] + j];
            acc[q].fma(df{a.x, a.y}, df{b.x, b.y});
          }
        }
      }
    }
  }
  // merge the slices of each output (slice 0 adds the others' sums)
  if (S > 1) {
    __syncthreads();
    red[tid] = make_float2(acc[0].s, acc[0].e);
    __syncthreads();
    if (sl == 0 && nq > 0) {
      df v = acc[0].value();
      for (int k = 1; k < S; ++k) {
        const float2 w = red[tid + k];
        v = df_add(v, df{w.x, w.y});
      }
      acc[0].s = v.h;
      acc[0].e = v.l;
    }
  }
  if (sl == 0) {
#pragma unroll
    for (int q = 0; q < kCbOut; ++q) {
      if (q < nq) {
        const int o = o0 + q * (kCbThreads / S);
        const int r = o / nmax, n = o - r * nmax;
        out[((size_t)s * nrow + r0 + r) * nmax + n] = (double)acc[q].s + (double)acc[q].e;
      }
    }
  }
}

static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

template <typename GT>
static int contract_batched(const float2* efp_df, const GT* G, int nsnap, int lmax, int nmax, int numr, double* out,
                            cudaStream_t st) {
  XT_REQUIRE((2 * lmax + 1) * nmax <= kCbOut * kCbThreads,
             "the batched contraction supports (2 lmax + 1) nmax <= %d", kCbOut * kCbThreads);
  const size_t smem = (size_t)(2 * lmax + 1 + nmax) * kCbPitch * sizeof(float2);
  static size_t attr = 0;
  if (smem > 48 * 1024 && smem > attr) {
    XT_CUDA(cudaFuncSetAttribute(k_sph_contract_batched_df<GT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
    attr = smem;
  }
  k_sph_contract_batched_df<GT><<<dim3((unsigned)nsnap, (unsigned)(lmax + 1)), kCbThreads, smem, st>>>(
      efp_df, G, lmax, nmax, numr, out);
  XT_CHECK_LAUNCH("k_sph_contract_batched_df");
  return XT_OK;
}

int launch_sph_contract_batched(const float2* efp_df, const double* G, int nsnap, int lmax, int nmax, int numr,
                                double* out, cudaStream_t st) {
  return contract_batched(efp_df, G, nsnap, lmax, nmax, numr, out, st);
}

int launch_sph_contract_batched(const float2* efp_df, const float2* G, int nsnap, int lmax, int nmax, int numr,
                                double* out, cudaStream_t st) {
  return contract_batched(efp_df, G, nsnap, lmax, nmax, numr, out, st);
}

}  // namespace xt

using namespace xt;

extern "C" {

size_t xt_sph_batched_workspace(void* handle, int nsnap, long long n_total, int chunk) {
  SphTab<double> d;
  if (!sph_tabs(handle, &d, nullptr) || nsnap <= 0 || chunk <= 0) return 0;
  const size_t nrow = (size_t)(d.lmax + 1) * (d.lmax + 1);
  const size_t maxitems = (size_t)(n_total / chunk + nsnap + 1) * 8;
  return al256((size_t)nsnap * nrow * d.numr * sizeof(double)) + al256(maxitems * sizeof(BatchItem)) +
         al256(64 * sizeof(int)) + al256(sizeof(int));
}

int xt_sph_accumulate_batched(void* handle, const float* xyzm, const long long* offsets_host, int nsnap,
                              int no_odd, int chunk, int threads, double* expcoef_out, void* workspace,
                              size_t workspace_bytes, void* stream) {
  SphTab<double> d;
  SphTab<float> f;
  XT_REQUIRE(sph_tabs(handle, &d, &f), "NULL table handle");
  XT_REQUIRE(nsnap > 0 && offsets_host && expcoef_out, "need nsnap > 0, host offsets and an output");
  XT_REQUIRE(chunk >= 256, "chunk must be >= 256 particles");
  XT_REQUIRE(threads == 128 || threads == 256 || threads == 512 || threads == 768 || threads == 1024,
             "threads must be 128, 256, 512, 768 or 1024");
  XT_REQUIRE(d.lmax <= 8, "the batched path supports lmax <= 8");
  const long long n_total = offsets_host[nsnap] - offsets_host[0];
  XT_REQUIRE(n_total >= 0 && offsets_host[0] == 0, "offsets must start at 0 and be non-decreasing");
  for (int s = 0; s < nsnap; ++s) XT_REQUIRE(offsets_host[s + 1] >= offsets_host[s], "offsets must be non-decreasing");
  XT_REQUIRE(n_total == 0 || xyzm, "NULL particle stream");
  XT_REQUIRE(((uintptr_t)xyzm & 15) == 0, "xyzm must be 16-byte aligned (float4 per particle)");
  const size_t need = xt_sph_batched_workspace(handle, nsnap, n_total, chunk);
  if (!workspace || workspace_bytes < need) {
    set_error("workspace of %zu bytes needed, %zu given", need, workspace_bytes);
    return XT_ERR_WORKSPACE;
  }
  // node parts: each part's shared grid (all rows x its nodes + 1) must fit
  // in 200 KB of shared memory
  const int nrow = (d.lmax + 1) * (d.lmax + 1);
  const size_t smem_cap = 200 * 1024;
  const int nodes_per_part = (int)(smem_cap / ((size_t)nrow * sizeof(float))) - 1;
  XT_REQUIRE(nodes_per_part >= 8, "lmax %d too large for the shared-memory grid", d.lmax);
  const int nint = d.numr - 1;                          // interpolation intervals i = 0..numr-2
  const int nparts = (nint + nodes_per_part - 1) / nodes_per_part;
  XT_REQUIRE(nparts <= 63, "too many node parts");
  std::vector<int> part_rows(nparts + 1);               // interval bounds ilo_k
  for (int k = 0; k <= nparts; ++k) part_rows[k] = (int)((long long)nint * k / nparts);
  int max_span = 0;
  for (int k = 0; k < nparts; ++k) max_span = std::max(max_span, part_rows[k + 1] - part_rows[k] + 1);
  const int max_rows = nrow;
  std::vector<BatchItem> items;
  for (int s = 0; s < nsnap; ++s)
    for (long long b = offsets_host[s]; b < offsets_host[s + 1]; b += chunk)
      for (int k = 0; k < nparts; ++k)
        items.push_back(BatchItem{s, k, b, std::min(b + (long long)chunk, offsets_host[s + 1])});
  const size_t maxitems = (size_t)(n_total / chunk + nsnap + 1) * 8;
  XT_REQUIRE(items.size() <= maxitems, "internal: work item table overflow");
  cudaStream_t st = as_stream(stream);
  char* ws = static_cast<char*>(workspace);
  double* G = reinterpret_cast<double*>(ws);
  size_t o = al256((size_t)nsnap * nrow * d.numr * sizeof(double));
  BatchItem* ditems = reinterpret_cast<BatchItem*>(ws + o);
  o += al256(maxitems * sizeof(BatchItem));
  int* dparts = reinterpret_cast<int*>(ws + o);
  o += al256(64 * sizeof(int));
  int* counter = reinterpret_cast<int*>(ws + o);
  XT_CUDA(cudaMemsetAsync(G, 0, (size_t)nsnap * nrow * d.numr * sizeof(double), st));
  XT_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), st));
  if (!items.empty()) {
    XT_CUDA(cudaMemcpyAsync(ditems, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice, st));
    XT_CUDA(cudaMemcpyAsync(dparts, part_rows.data(), part_rows.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    const size_t smem = (size_t)max_rows * max_span * sizeof(float);
    int dev = 0, nsm = 0;
    XT_CUDA(cudaGetDevice(&dev));
    XT_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    int rc = with_lcap(d.lmax, [&](auto lc) -> int {
      constexpr int LC = decltype(lc)::value;
      {
        const int per_sm = resident_blocks_full_carveout((const void*)k_sph_batched<LC>, threads, smem);
        if (per_sm < 1) {
          set_error("k_sph_batched cannot run %d threads with %zu bytes of shared memory", threads, smem);
          return XT_ERR_ARG;
        }
        const int grid = nsm * per_sm;
        k_sph_batched<LC><<<grid, threads, smem, st>>>(f, reinterpret_cast<const float4*>(xyzm), ditems,
                                                      (int)items.size(), counter, dparts, no_odd, G);
        return XT_OK;
      }
    });
    if (rc) return rc;
    XT_CHECK_LAUNCH("k_sph_batched");
  }
  const float2* efp_df = nullptr;
  XT_REQUIRE(sph_efp_df(handle, &efp_df), "NULL table handle");
  return launch_sph_contract_batched(efp_df, G, nsnap, d.lmax, d.nmax, d.numr, expcoef_out, st);
}

}  // extern "C"
