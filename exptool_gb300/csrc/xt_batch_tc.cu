// Batched spherical accumulation on the 5th-generation tensor cores.
//
// The same sums as k_sph_batched (xt_batch.cu), the coefficient time series
// spheresl.compute_coefficients (spheresl.py:439-475, accumulation loop
// :598-654) would produce snapshot by snapshot, written as dense products.
// The radial table interpolation is linear in the node values, so
//   expcoef[s, row, n] = sum_node ef'[l(row), n, node] G[s, row, node],
//   G[s, row, node]    = sum_p W[p, node] A[p, row],
// with A[p, row] = P_l^m(cos th_p) {1, cos m phi_p, sin m phi_p} (the
// angular basis values of particle p, the normalisation fact[l][m] applied
// in FP64 to G; a BF16 rounding of it would bias every particle alike) and
// W[p, node] its two non-zero
// interpolation weights -4 pi m_p plerp_p {x1_p, x2_p} on nodes i_p, i_p + 1
// (the nodal hat-function basis of the table interpolation).  G is a
// particles x basis-terms product: for a window of 128 consecutive nodes,
//   D[node, row] = sum_p W^T[node, p] A[p, row]
// is one tcgen05.mma chain with M = 128 nodes, N = rows (padded to a multiple
// of 16), K = particles, BF16 operands and FP32 accumulation in tensor memory.
//
// Pipeline (one call, all snapshots):
//   1. k_bt_hist: counts per (sorting chunk, window of 127 intervals) of the
//      particles' node intervals (recomputed bit for bit by the scatter and
//      the products, so nothing per particle is stored);
//   2. k_bt_offsets, k_bt_buckets, k_bt_items: per-chunk offsets inside each
//      (snapshot, window) bucket, bucket bases, and work items (bucket pieces
//      of at most `chunk` particles);
//   3. k_bt_scatter: counting sort of the particles by (snapshot, window);
//   4. k_sph_batched_tc: persistent; a CTA takes an item, builds the W^T and
//      A tiles of 128 particles per K-tile in shared memory (one particle per
//      thread, BF16; W^T K-major, A MN-major), one thread issues the MMAs
//      and commits them to the stage's mbarrier while the next stage is
//      built; at the item's end the accumulator (128 nodes x rows, FP32) is
//      read from tensor memory into a per-item partial;
//   5. k_bt_reduce: exact double-float sum of the partials per (snapshot,
//      row, node), in a fixed order (the window boundary node takes both
//      windows' shares), times fact[l][m];
//   6. k_sph_contract_batched_df: contraction with the radial tables in
//      double-float arithmetic (FP64-level accuracy on the FP32 pipe).
// Waits are bounded: a timeout sets the error flag read by
// xt_sph_batched_tc_status, waits once more for the MMAs in flight, frees the
// tensor memory and returns.
#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include <cuda_bf16.h>

#include "xt_df.cuh"
#include "xt_internal.cuh"
#include "xt_launch.cuh"
#include "xt_tc.cuh"

namespace xt {

constexpr int BT_M = 128;                   // nodes per window tile (tensor-memory lanes)
constexpr int BT_NODES = BT_M - 1;          // interpolation intervals per window
constexpr int BT_KT = 128;                  // particles per K-tile (one per thread)
constexpr int BT_THREADS = 128;
constexpr int BT_LBO = 128;                 // bytes between core matrices along K
constexpr int BT_SBO = (BT_KT / 8) * 128;   // bytes between 8-row groups
constexpr int BT_A_BYTES = BT_M * BT_KT * 2;
constexpr int BT_SORT_CHUNK = 4096;         // particles per sorting chunk
constexpr int BT_MAXWIN = 64;               // windows per snapshot (numr <= 64 * 127 + 1)
constexpr float BT_FOUR_PI = 12.566370614359172f;

struct BtChunk {
  int snap;
  int pad;
  long long begin, end;
};

struct BtItem {
  int bucket, snap, win, pad;
  long long begin, end;
};

struct BtArgs {
  SphTab<float> T;
  const float4* sorted;
  const BtItem* items;
  const int* nitems;
  int* counter;
  float* partial;       // [item][nrow][128]
  int* err;
  int nrow, no_odd;
};

__device__ __forceinline__ int bt_off(int row, int k) {
  return (row >> 3) * BT_SBO + (k >> 3) * BT_LBO + (row & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ void bt_st(unsigned char* tile, int row, int k, float v) {
  *reinterpret_cast<__nv_bfloat16*>(tile + bt_off(row, k)) = __float2bfloat16_rn(v);
}

// Radius, mapped radius and interpolation interval of a particle.  The
// counting sort (k_bt_hist, k_bt_scatter) and the products (k_sph_batched_tc)
// each compute them from the particle, so every operation is an explicitly
// rounded intrinsic (no multiply-add contraction left to the compiler) and
// the three kernels get the same bits: the interval that put a particle into
// a window is the one its weights are taken on.
__device__ __forceinline__ float bt_radius(float4 q) {
  const float r = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(q.x, q.x), __fmul_rn(q.y, q.y)), __fmul_rn(q.z, q.z)));
  return (r >= 1.0e-10f) ? r : 1.0e-10f;
}

// compatibility.r_to_xi (compatibility.py:16-36) for r > 0, clamped to the
// table as sph_bins does (spheresl.py:121-131).
__device__ __forceinline__ float bt_xi(const SphTab<float>& T, float r) {
  float x;
  if (T.cmap == 1) {
    const float u = __fmul_rn(r, T.inv_scale);
    x = __fdiv_rn(__fsub_rn(u, 1.f), __fadd_rn(u, 1.f));
    x = fminf(fmaxf(x, -1.f), 1.f - 1.0e-8f);
  } else if (T.cmap == 2) {
    x = fminf(fmaxf(logf(r), T.lo), T.hi);
  } else {
    x = r;
  }
  return x;
}

// Interpolation interval of mapped radius x: the node index of sph_bins
// (spheresl.py:121-131).
__device__ __forceinline__ int bt_interval(const SphTab<float>& T, float x) {
  float fi = floorf(__fmul_rn(__fsub_rn(x, T.xi0), T.inv_dxi));
  if (!(fi >= 0.f)) fi = 0.f;
  if (fi > (float)(T.numr - 2)) fi = (float)(T.numr - 2);
  return (int)fi;
}

// ------------------------------------------------------------------ sort
// Exclusive scan over a block of 256 threads; *total receives the block sum.
__device__ __forceinline__ int bt_block_scan(int v, int* wsum, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  if (lane == 31) wsum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    const int t = lane < 8 ? wsum[lane] : 0;
    int u = t;
#pragma unroll
    for (int d = 1; d < 8; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, u, d);
      if (lane >= d) u += y;
    }
    if (lane < 8) wsum[lane] = u - t;
    if (lane == 7) wsum[8] = u;
  }
  __syncthreads();
  const int r = x - v + wsum[wid];
  *total = wsum[8];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(256) k_bt_hist(SphTab<float> T, const float4* __restrict__ xyzm,
                                                 const BtChunk* __restrict__ chunks, int nchunk, int nwin,
                                                 int* __restrict__ ccount) {
  __shared__ int cnt[BT_MAXWIN];
  for (int c = blockIdx.x; c < nchunk; c += gridDim.x) {
    for (int w = threadIdx.x; w < nwin; w += blockDim.x) cnt[w] = 0;
    __syncthreads();
    const BtChunk C = chunks[c];
    for (long long p = C.begin + threadIdx.x; p < C.end; p += blockDim.x) {
      const int i = bt_interval(T, bt_xi(T, bt_radius(xyzm[p])));
      atomicAdd(&cnt[i / BT_NODES], 1);
    }
    __syncthreads();
    for (int w = threadIdx.x; w < nwin; w += blockDim.x) ccount[(size_t)c * nwin + w] = cnt[w];
    __syncthreads();
  }
}

// One block per snapshot: offsets of each chunk inside its (snapshot, window)
// bucket and the bucket sizes.
__global__ void __launch_bounds__(256) k_bt_offsets(const int* __restrict__ cfirst, int nwin,
                                                    const int* __restrict__ ccount, int* __restrict__ coff,
                                                    long long* __restrict__ bsize) {
  __shared__ int wsum[9];
  const int s = blockIdx.x;
  const int c0 = cfirst[s], c1 = cfirst[s + 1];
  for (int w = 0; w < nwin; ++w) {
    long long carry = 0;
    for (int base = c0; base < c1; base += blockDim.x) {
      const int c = base + threadIdx.x;
      const int v = c < c1 ? ccount[(size_t)c * nwin + w] : 0;
      int tot;
      const int ex = bt_block_scan(v, wsum, &tot);
      if (c < c1) coff[(size_t)c * nwin + w] = (int)carry + ex;
      carry += tot;
    }
    if (threadIdx.x == 0) bsize[(size_t)s * nwin + w] = carry;
  }
}

// One block: bucket bases (particle offsets in the sorted stream) and the
// first work item of every bucket.
__global__ void __launch_bounds__(256) k_bt_buckets(const long long* __restrict__ bsize, int nb, int chunk,
                                                    long long* __restrict__ bbase, int* __restrict__ ifirst,
                                                    int* __restrict__ nitems) {
  __shared__ int wsum[9];
  __shared__ long long tile[256];
  __shared__ long long carry_p;
  int carry_i = 0;
  if (threadIdx.x == 0) carry_p = 0;
  for (int base = 0; base < nb; base += blockDim.x) {
    const int b = base + threadIdx.x;
    const long long sz = b < nb ? bsize[b] : 0;
    int tot;
    const int ex = bt_block_scan((int)((sz + chunk - 1) / chunk), wsum, &tot);
    tile[threadIdx.x] = sz;
    __syncthreads();
    if (threadIdx.x == 0) {            // particle offsets exceed int: a serial scan of the tile
      long long acc = carry_p;
      for (int k = 0; k < (int)blockDim.x; ++k) {
        const long long t = tile[k];
        tile[k] = acc;
        acc += t;
      }
      carry_p = acc;
    }
    __syncthreads();
    if (b < nb) {
      bbase[b] = tile[threadIdx.x];
      ifirst[b] = carry_i + ex;
    }
    carry_i += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    ifirst[nb] = carry_i;
    *nitems = carry_i;
  }
}

__global__ void k_bt_items(const long long* __restrict__ bsize, const long long* __restrict__ bbase,
                           const int* __restrict__ ifirst, int nb, int nwin, int chunk, BtItem* __restrict__ items) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
    const long long sz = bsize[b], b0 = bbase[b];
    int it = ifirst[b];
    for (long long o = 0; o < sz; o += chunk, ++it)
      items[it] = BtItem{b, b / nwin, b % nwin, 0, b0 + o, b0 + (o + chunk < sz ? o + chunk : sz)};
  }
}

__global__ void __launch_bounds__(256) k_bt_scatter(SphTab<float> T, const float4* __restrict__ xyzm,
                                                    const BtChunk* __restrict__ chunks, int nchunk, int nwin,
                                                    const int* __restrict__ coff, const long long* __restrict__ bbase,
                                                    long long n_total, float4* __restrict__ sorted,
                                                    int* __restrict__ err) {
  __shared__ int cnt[BT_MAXWIN];
  for (int c = blockIdx.x; c < nchunk; c += gridDim.x) {
    for (int w = threadIdx.x; w < nwin; w += blockDim.x) cnt[w] = 0;
    __syncthreads();
    const BtChunk C = chunks[c];
    for (long long p = C.begin + threadIdx.x; p < C.end; p += blockDim.x) {
      const float4 q = xyzm[p];
      const int w = bt_interval(T, bt_xi(T, bt_radius(q))) / BT_NODES;
      const int slot = atomicAdd(&cnt[w], 1);
      const long long dst = bbase[(size_t)C.snap * nwin + w] + coff[(size_t)c * nwin + w] + slot;
      if (dst >= 0 && dst < n_total) {
        sorted[dst] = q;
      } else {
        atomicExch(err, 2);
      }
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------ tensor-core products
// Operand tiles of one stage (K = 128 particles, one per thread):
//  * the angular values A^T (N = NPAD rows x K particles) first, in the
//    MN-major canonical layout: element (n, k) at (k >> 3) * BSK + (n >> 3) * 128
//    + (k & 7) * 16 + (n & 7) * 2, so a thread stores 8 consecutive rows of its
//    particle as one 16-byte word (conflict-free across the warp);
//  * the weights W^T (M = 128 nodes x K particles) after it, K-major: element
//    (node, k) at bt_off(node, k).
// A wrongly read stride could only reach into the stage's own W^T tile: the
// angular tile comes first.
template <int NPAD>
struct BtTile {
  static constexpr int BSK = (NPAD / 8) * 128;        // bytes between 8-particle groups (K direction)
  static constexpr int B_BYTES = NPAD * BT_KT * 2;
  static constexpr int STAGE = B_BYTES + BT_A_BYTES;
};

// Associated Legendre P_l^m(x) by the recurrences of legendre() (spheresl.py:
// 664-700) for a finite x in [-1, 1], where every value is finite.
template <int LCAP>
__device__ __forceinline__ void bt_legendre(float x, float* P) {
  const float somx2 = sqrtf((1.f - x) * (1.f + x));
  P[0] = 1.f;
  float pll = 1.f, fact = 1.f;
#pragma unroll
  for (int m = 1; m <= LCAP; ++m) {
    pll *= -fact * somx2;
    P[tri(m, m)] = pll;
    fact += 2.f;
  }
#pragma unroll
  for (int m = 0; m < LCAP; ++m) {
    float pl2 = P[tri(m, m)];
    float pl1 = x * (float)(2 * m + 1) * pl2;
    P[tri(m + 1, m)] = pl1;
#pragma unroll
    for (int l = m + 2; l <= LCAP; ++l) {
      const float v = (x * (float)(2 * l - 1) * pl1 - (float)(l + m - 1) * pl2) * (1.f / (float)(l - m));
      P[tri(l, m)] = v;
      pl2 = pl1;
      pl1 = v;
    }
  }
}

// Two threads per particle: the angular rows are ordered by the parity of m,
// the even orders (m = 0, 2, ...) in the first 8 * G0 columns of the tile and
// the odd ones after them, each half a whole number of 8-row groups, so each
// thread of a pair stores its own 16-byte row chunks.  Within a half: for each
// m, the cosine rows l = m..LCAP, then the sine rows.  row[slot] is the
// coefficient row l^2 (m = 0), l^2 + 2m - 1 (cos) or l^2 + 2m (sin), -1 for
// padding.
template <int LCAP>
struct BtPerm {
  static constexpr int count(int parity) {
    int c = 0;
    for (int m = parity; m <= LCAP; m += 2) c += m == 0 ? LCAP + 1 : 2 * (LCAP - m + 1);
    return c;
  }
  static constexpr int G0 = (count(0) + 7) / 8, G1 = (count(1) + 7) / 8;
  int row[8 * (G0 + G1)];
  constexpr BtPerm() : row() {
    for (int s = 0; s < 8 * (G0 + G1); ++s) row[s] = -1;
    for (int h = 0; h < 2; ++h) {
      int slot = h ? 8 * G0 : 0;
      for (int m = h; m <= LCAP; m += 2) {
        for (int l = m; l <= LCAP; ++l) row[slot++] = l * l + (m == 0 ? 0 : 2 * m - 1);
        if (m > 0)
          for (int l = m; l <= LCAP; ++l) row[slot++] = l * l + 2 * m;
      }
    }
  }
};

// The angular values of one half (H = 0: even m, H = 1: odd m) in the slot
// order of BtPerm, from the recurrences of bt_legendre.
template <int LCAP, int H>
__device__ __forceinline__ void bt_half_values(float x, float somx2, const float* cm, const float* sn, int lmax,
                                               int no_odd, float* v) {
  float pmm[LCAP + 1];
  pmm[0] = 1.f;
  float fact = 1.f;
#pragma unroll
  for (int m = 1; m <= LCAP; ++m) {
    pmm[m] = pmm[m - 1] * (-fact * somx2);
    fact += 2.f;
  }
  int slot = 0;
#pragma unroll
  for (int m = H; m <= LCAP; m += 2) {
    float Pl[LCAP + 2];
    Pl[m] = pmm[m];
    if (m + 1 <= LCAP) Pl[m + 1] = x * (float)(2 * m + 1) * pmm[m];
#pragma unroll
    for (int l = m + 2; l <= LCAP; ++l)
      Pl[l] = (x * (float)(2 * l - 1) * Pl[l - 1] - (float)(l + m - 1) * Pl[l - 2]) * (1.f / (float)(l - m));
#pragma unroll
    for (int l = m; l <= LCAP; ++l) {
      const bool on = l <= lmax && !(no_odd && (l & 1));
      const float pv = on ? Pl[l] : 0.f;
      if (m == 0) {
        v[slot + (l - m)] = pv;
      } else {
        v[slot + (l - m)] = pv * cm[m];
        v[slot + (LCAP - m + 1) + (l - m)] = pv * sn[m];
      }
    }
    slot += m == 0 ? LCAP + 1 : 2 * (LCAP - m + 1);
  }
}

template <int LCAP, int NPAD, int STAGES, int SPLIT>
__global__ void __launch_bounds__(BT_THREADS * SPLIT, SPLIT == 2 ? 3 : 1) k_sph_batched_tc(BtArgs a) {
  using TL = BtTile<NPAD>;
  using PM = BtPerm<LCAP>;
  static_assert(SPLIT == 1 || 8 * (PM::G0 + PM::G1) <= NPAD, "split rows exceed the padded tile");
  constexpr int NCOLS = NPAD <= 32 ? 32 : (NPAD <= 64 ? 64 : (NPAD <= 128 ? 128 : 256));
  constexpr int NT = (LCAP + 1) * (LCAP + 2) / 2;
  constexpr int NROW = (LCAP + 1) * (LCAP + 1);
  static_assert(NROW <= NPAD, "rows exceed the padded tile");
  extern __shared__ __align__(1024) unsigned char sm[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + STAGES * TL::STAGE);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + STAGES);
  int* s_item = reinterpret_cast<int*>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int kp = tid & (BT_KT - 1);          // this thread's particle slot of a K-tile
  const int half = SPLIT == 2 ? tid / BT_KT : 0;
  const SphTab<float>& T = a.T;
  const int lmax = T.lmax;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid < STAGES) mbar_init(smem_u32(bars + tid));
  // operand tiles start at zero: padded angular rows and the weight rows no
  // particle touches stay zero
  for (int o = tid * 16; o < STAGES * TL::STAGE; o += BT_THREADS * SPLIT * 16)
    *reinterpret_cast<uint4*>(sm + o) = make_uint4(0u, 0u, 0u, 0u);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // kind::f16, D F32, A (weights) K-major, B (angular) MN-major (bit 16)
  const uint32_t idesc = tc_idesc(BT_M, NPAD) | (1u << 16);
  const int nitems = *a.nitems;
  // byte offset of this thread's angular column in a stage's angular tile
  const int kofs = (kp >> 3) * TL::BSK + (kp & 7) * 16;
  int prev_row[STAGES];
#pragma unroll
  for (int s = 0; s < STAGES; ++s) prev_row[s] = -1;
  long long g = 0;          // K-tiles issued by this CTA (stage g % STAGES)
  bool ok = true;           // block-uniform: every failure test is a __syncthreads_or

  for (;;) {
    if (tid == 0) *s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const int it = *s_item;
    if (it >= nitems) break;
    const BtItem I = a.items[it];
    const int wbase = I.win * BT_NODES;
    const long long ntile = (I.end - I.begin + BT_KT - 1) / BT_KT;
    // this thread's particle of the next K-tile is loaded one tile ahead
    float4 qn = make_float4(0.f, 0.f, 0.f, 0.f);
    if (I.begin + kp < I.end) qn = a.sorted[I.begin + kp];
    for (long long t = 0; t < ntile; ++t, ++g) {
      const float4 q = qn;
      const bool have = I.begin + t * BT_KT + kp < I.end;
      const long long pn = I.begin + (t + 1) * BT_KT + kp;
      if (pn < I.end) qn = a.sorted[pn];
      // this particle's values, computed before its stage is free
      uint32_t pk[NPAD / 2];
#pragma unroll
      for (int k = 0; k < NPAD / 2; ++k) pk[k] = 0u;
      float w0 = 0.f, w1 = 0.f;
      int li = -1;
      if (have) {
        const float r = bt_radius(q);
        // interpolation weights on the interval that sorted the particle
        // into this window (spheresl.py:121-143)
        const float x = bt_xi(T, r);
        const int i = bt_interval(T, x);
        const float x2 = (x - T.xi[i]) * T.inv_dxi, x1 = 1.f - x2;
        const float plerp = x1 * T.p0[i] + x2 * T.p0[i + 1];
        const float base = -BT_FOUR_PI * q.w * plerp;
        w0 = x1 * base;
        w1 = x2 * base;
        li = i - wbase;
        const float costh = q.z / r;
        float c1, s1;
        unit_phi(q.x, q.y, c1, s1);
        float cm[LCAP + 1], sn[LCAP + 1];
        multiples<float, LCAP>(c1, s1, LCAP, cm, sn);
        if constexpr (SPLIT == 1) {
          float P[NT];
          bt_legendre<LCAP>(costh, P);
          float v[NPAD];
#pragma unroll
          for (int k = 0; k < NPAD; ++k) v[k] = 0.f;
          // the normalisation fact[l][m] is applied in FP64 by k_bt_reduce: a
          // BF16 rounding of it would bias every particle alike
#pragma unroll
          for (int l = 0; l <= LCAP; ++l) {
            const bool on = l <= lmax && !(a.no_odd && (l & 1));   // rows of odd l stay zero under no_odd
#pragma unroll
            for (int m = 0; m <= l; ++m) {
              const float pv = on ? P[tri(l, m)] : 0.f;
              if (m == 0) {
                v[l * l] = pv;
              } else {
                v[l * l + 2 * m - 1] = pv * cm[m];
                v[l * l + 2 * m] = pv * sn[m];
              }
            }
          }
#pragma unroll
          for (int k = 0; k < NPAD / 2; ++k) {
            __nv_bfloat162 b2 = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
            pk[k] = *reinterpret_cast<uint32_t*>(&b2);
          }
        } else {
          // this thread's half of the rows (warp-uniform branch)
          const float somx2 = sqrtf((1.f - costh) * (1.f + costh));
          constexpr int NV = 8 * (PM::G0 > PM::G1 ? PM::G0 : PM::G1);
          float v[NV];
#pragma unroll
          for (int k = 0; k < NV; ++k) v[k] = 0.f;
          if (half == 0) bt_half_values<LCAP, 0>(costh, somx2, cm, sn, lmax, a.no_odd, v);
          else bt_half_values<LCAP, 1>(costh, somx2, cm, sn, lmax, a.no_odd, v);
#pragma unroll
          for (int k = 0; k < NV / 2; ++k) {
            __nv_bfloat162 b2 = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
            pk[k] = *reinterpret_cast<uint32_t*>(&b2);
          }
        }
      }
      const int st = (int)(g % STAGES);
      unsigned char* Bt = sm + st * TL::STAGE;
      unsigned char* At = Bt + TL::B_BYTES;
      // the MMAs that last read this stage (K-tile g - STAGES) must be done
      bool lf = false;
      if (tid == 0 && g >= STAGES) lf = !mbar_wait(smem_u32(bars + st), (uint32_t)(((g / STAGES) - 1) & 1));
      if (__syncthreads_or(lf)) {
        ok = false;
        break;
      }
      int pr = -1;
#pragma unroll
      for (int s = 0; s < STAGES; ++s)
        if (s == st) pr = prev_row[s];
      int nr = -1;
      if (half == 0) {                           // the weights: one thread per particle
        if (pr >= 0) {
          *reinterpret_cast<__nv_bfloat16*>(At + bt_off(pr, kp)) = __float2bfloat16_rn(0.f);
          *reinterpret_cast<__nv_bfloat16*>(At + bt_off(pr + 1, kp)) = __float2bfloat16_rn(0.f);
        }
        if (have) {
          if (li >= 0 && li < BT_NODES) {
            bt_st(At, li, kp, w0);
            bt_st(At, li + 1, kp, w1);
            nr = li;
          } else {
            atomicExch(a.err, 3);
          }
        }
      }
      // the angular column: chunks of 8 rows (rows no chunk covers are zero
      // from the start and never written); zeros for a missing particle (a
      // stale non-finite value would survive zero weights)
      if constexpr (SPLIT == 1) {
#pragma unroll
        for (int c = 0; c < (NROW + 7) / 8; ++c)
          *reinterpret_cast<uint4*>(Bt + kofs + c * 128) =
              make_uint4(pk[4 * c], pk[4 * c + 1], pk[4 * c + 2], pk[4 * c + 3]);
      } else {
        const int g0 = half ? PM::G0 : 0, ng = half ? PM::G1 : PM::G0;
#pragma unroll
        for (int c = 0; c < (PM::G0 > PM::G1 ? PM::G0 : PM::G1); ++c)
          if (c < ng)
            *reinterpret_cast<uint4*>(Bt + kofs + (g0 + c) * 128) =
                make_uint4(pk[4 * c], pk[4 * c + 1], pk[4 * c + 2], pk[4 * c + 3]);
      }
#pragma unroll
      for (int s = 0; s < STAGES; ++s)
        if (s == st) prev_row[s] = nr;
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
      tc_fence_after();
      if (tid == 0) {
        const uint32_t ab = smem_u32(At), bb = smem_u32(Bt);
#pragma unroll
        for (int kk = 0; kk < BT_KT / 16; ++kk)
          tc_mma(tmem, tc_desc(ab + kk * 2 * BT_LBO, BT_LBO, BT_SBO),
                 tc_desc(bb + kk * 2 * TL::BSK, TL::BSK, 128), idesc, (t > 0 || kk > 0) ? 1u : 0u);
        tc_commit(smem_u32(bars + st));
      }
    }
    if (!ok) break;
    // the item's sums: wait for its last MMAs, read the accumulator rows
    const int lst = (int)((g - 1) % STAGES);
    bool lf = false;
    if (tid == 0) lf = !mbar_wait(smem_u32(bars + lst), (uint32_t)(((g - 1) / STAGES) & 1));
    if (__syncthreads_or(lf)) {
      ok = false;
      break;
    }
    tc_fence_after();
    // a warp reads its quarter's lanes; with two threads per particle the
    // second warpgroup reads the second half of the columns
    const uint32_t trow = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    float* dst = a.partial + (size_t)it * a.nrow * BT_M + 32 * (warp & 3) + (tid & 31);
    if constexpr (SPLIT == 1) {
#pragma unroll 1
      for (int c16 = 0; c16 < NPAD / 16; ++c16) {
        float v[16];
        tc_ld16(trow + 16 * c16, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int row = 16 * c16 + j;
          if (row < a.nrow) dst[(size_t)row * BT_M] = v[j];
        }
      }
    } else {
      constexpr PM perm{};
      constexpr int HALF = NPAD / 2;
      static_assert(HALF % 16 == 0, "column halves of whole 16-column loads");
#pragma unroll
      for (int c16 = 0; c16 < HALF / 16; ++c16) {
        float v[16];
        const int col0 = (warp >> 2) * HALF + 16 * c16;
        tc_ld16(trow + col0, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int c0 = 16 * c16 + j;       // column within this warpgroup's half
          const int row = (warp >> 2) ? (HALF + c0 < 8 * (PM::G0 + PM::G1) ? perm.row[HALF + c0] : -1)
                                      : (c0 < 8 * (PM::G0 + PM::G1) ? perm.row[c0] : -1);
          if (row >= 0 && row < a.nrow) dst[(size_t)row * BT_M] = v[j];
        }
      }
    }
    tc_fence_before();
    __syncthreads();
  }
  // after a wait gave up, the MMAs still in flight finish (bounded) before the
  // tensor memory is released
  if (!ok && g > 0 && tid == 0) mbar_wait(smem_u32(bars + (int)((g - 1) % STAGES)), (uint32_t)(((g - 1) / STAGES) & 1));
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && !ok) atomicExch(a.err, 1);
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOLS) : "memory");
  }
}

// G[s, row, node] = fact[l][m] times the sum of the partials of the windows
// holding the node, in item order.  Node 127 w (w >= 1) is lane 0 of window w
// and lane 127 of window w - 1.  The FP32 partials are summed exactly into a
// double-float (TwoSum on the FP32 pipe; GB300's FP64 pipe is slow), times
// fact as a double-float product, and stored as the (hi, lo) pair the
// double-float contraction reads.  One block per (snapshot, row), threads
// over the nodes.
__global__ void __launch_bounds__(256) k_bt_reduce(const float* __restrict__ partial, const int* __restrict__ ifirst,
                                                   const double* __restrict__ fact, int lmax, int nsnap, int nrow,
                                                   int numr, int nwin, float2* __restrict__ G) {
  for (long long sr = blockIdx.x; sr < (long long)nsnap * nrow; sr += gridDim.x) {
    const int row = (int)(sr % nrow), s = (int)(sr / nrow);
    int l = 0;
    while ((l + 1) * (l + 1) <= row) ++l;
    const int m = (row - l * l + 1) >> 1;            // row l^2 (m = 0), l^2 + 2m - 1 (cos), l^2 + 2m (sin)
    const df f = df_from(fact[l * (lmax + 1) + m]);
    for (int node = threadIdx.x; node < numr; node += blockDim.x) {
      const int w = node / BT_NODES, lane = node - w * BT_NODES;
      float hi = 0.f, lo = 0.f;
      auto add = [&](float x) {
        const float t = __fadd_rn(hi, x);
        const float v = __fsub_rn(t, hi);
        lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(t, v)), __fsub_rn(x, v)));
        hi = t;
      };
      if (w < nwin) {
        const int b = s * nwin + w;
        for (int it = ifirst[b]; it < ifirst[b + 1]; ++it) add(partial[((size_t)it * nrow + row) * BT_M + lane]);
      }
      if (lane == 0 && w >= 1) {
        const int b = s * nwin + w - 1;
        for (int it = ifirst[b]; it < ifirst[b + 1]; ++it) add(partial[((size_t)it * nrow + row) * BT_M + BT_NODES]);
      }
      const df v = df_mul(fast_two_sum(hi, lo), f);
      G[sr * numr + node] = make_float2(v.h, v.l);
    }
  }
}

static __device__ int g_bt_err;

static size_t bt_al(size_t b) { return (b + 255) & ~(size_t)255; }

struct BtLayout {
  size_t G, sorted, chunks, cfirst, ccount, coff, bsize, bbase, ifirst, items, partial, ctr, total;
  long long max_items;
  int nwin, nb;
  long long nchunk;
};

static BtLayout bt_layout(const SphTab<double>& d, int nsnap, long long n_total, long long nchunk, int chunk) {
  BtLayout L;
  const int nrow = (d.lmax + 1) * (d.lmax + 1);
  L.nwin = (d.numr - 2) / BT_NODES + 1;
  L.nb = nsnap * L.nwin;
  L.nchunk = nchunk;
  L.max_items = n_total / chunk + L.nb + 1;
  size_t o = 0;
  auto take = [&](size_t b) { const size_t at = o; o += bt_al(b); return at; };
  L.G = take((size_t)nsnap * nrow * d.numr * sizeof(float2));
  L.sorted = take((size_t)n_total * sizeof(float4));
  L.chunks = take((size_t)nchunk * sizeof(BtChunk));
  L.cfirst = take((size_t)(nsnap + 1) * sizeof(int));
  L.ccount = take((size_t)nchunk * L.nwin * sizeof(int));
  L.coff = take((size_t)nchunk * L.nwin * sizeof(int));
  L.bsize = take((size_t)L.nb * sizeof(long long));
  L.bbase = take((size_t)L.nb * sizeof(long long));
  L.ifirst = take((size_t)(L.nb + 1) * sizeof(int));
  L.items = take((size_t)L.max_items * sizeof(BtItem));
  L.partial = take((size_t)L.max_items * nrow * BT_M * sizeof(float));
  L.ctr = take(4 * sizeof(int));
  L.total = o;
  return L;
}

static long long bt_nchunk(const long long* off, int nsnap) {
  long long n = 0;
  for (int s = 0; s < nsnap; ++s) n += (off[s + 1] - off[s] + BT_SORT_CHUNK - 1) / BT_SORT_CHUNK;
  return n;
}

// CTAs of k_sph_batched_tc<LC, NPAD, STAGES, SPLIT> resident per SM: as many
// as the registers, the whole unified L1/shared storage as shared memory (the
// default carveout leaves one per SM) and the SM's 512 tensor-memory columns
// allow; 0 if none.
template <int LC, int NPAD, int STAGES, int SPLIT>
static int bt_residency() {
  constexpr size_t smem = (size_t)STAGES * BtTile<NPAD>::STAGE + STAGES * 8 + 8;
  constexpr int ncols = NPAD <= 32 ? 32 : (NPAD <= 64 ? 64 : (NPAD <= 128 ? 128 : 256));
  return resident_blocks_tmem((const void*)k_sph_batched_tc<LC, NPAD, STAGES, SPLIT>, BT_THREADS * SPLIT, smem,
                              ncols);
}

// Persistent launch of ctas_per_sm CTAs per SM (0: as many as are resident).
template <int LC, int NPAD, int STAGES, int SPLIT>
static int bt_launch_gemm(const BtArgs& A, int ctas_per_sm, cudaStream_t st) {
  constexpr size_t smem = (size_t)STAGES * BtTile<NPAD>::STAGE + STAGES * 8 + 8;
  int per_sm = bt_residency<LC, NPAD, STAGES, SPLIT>();
  XT_REQUIRE(per_sm >= 1, "k_sph_batched_tc does not fit on an SM with %zu bytes of shared memory", smem);
  if (ctas_per_sm > 0) per_sm = std::min(per_sm, ctas_per_sm);
  k_sph_batched_tc<LC, NPAD, STAGES, SPLIT><<<sm_count() * per_sm, BT_THREADS * SPLIT, smem, st>>>(A);
  XT_CHECK_LAUNCH("k_sph_batched_tc");
  return XT_OK;
}

// Dispatch on the threads per particle.
template <typename F>
static int bt_with_split(int split, F&& f) {
  if (split == 2) return f(std::integral_constant<int, 2>{});
  return f(std::integral_constant<int, 1>{});
}

// Dispatch on the pipeline depth.
template <int LC, int NPAD, typename F>
static int bt_with_stages(int stages, F&& f) {
  if (stages == 1) return f(std::integral_constant<int, 1>{});
  if (stages == 2) return f(std::integral_constant<int, 2>{});
  return f(std::integral_constant<int, 3>{});
}

}  // namespace xt

using namespace xt;

extern "C" {

size_t xt_sph_batched_tc_workspace(void* handle, int nsnap, const long long* offsets_host, int chunk) {
  SphTab<double> d;
  if (!sph_tabs(handle, &d, nullptr) || nsnap <= 0 || !offsets_host || chunk < BT_KT) return 0;
  const long long n_total = offsets_host[nsnap] - offsets_host[0];
  if (n_total < 0) return 0;
  return bt_layout(d, nsnap, n_total, bt_nchunk(offsets_host, nsnap), chunk).total;
}

int xt_sph_accumulate_batched_tc(void* handle, const float* xyzm, const long long* offsets_host, int nsnap,
                                 int no_odd, int chunk, int stages, int ctas_per_sm, int threads_per_particle,
                                 double* expcoef_out, void* workspace, size_t workspace_bytes, void* stream) {
  SphTab<double> d;
  SphTab<float> f;
  XT_REQUIRE(sph_tabs(handle, &d, &f), "NULL table handle");
  XT_REQUIRE(nsnap > 0 && offsets_host && expcoef_out, "need nsnap > 0, host offsets and an output");
  XT_REQUIRE(chunk >= BT_KT && chunk <= (1 << 30), "chunk must be in [%d, 2^30] particles", BT_KT);
  XT_REQUIRE(stages >= 1 && stages <= 3, "stages must be 1, 2 or 3");
  XT_REQUIRE(ctas_per_sm >= 0, "ctas_per_sm must be >= 0 (0: as many as are resident)");
  XT_REQUIRE(threads_per_particle == 1 || threads_per_particle == 2, "threads_per_particle must be 1 or 2");
  XT_REQUIRE(d.lmax <= 8, "the batched path supports lmax <= 8");
  XT_REQUIRE(d.numr >= 2 && (d.numr - 2) / BT_NODES + 1 <= BT_MAXWIN, "numr must be in [2, %d]",
             BT_MAXWIN * BT_NODES + 1);
  const long long n_total = offsets_host[nsnap] - offsets_host[0];
  XT_REQUIRE(n_total >= 0 && offsets_host[0] == 0, "offsets must start at 0 and be non-decreasing");
  for (int s = 0; s < nsnap; ++s) XT_REQUIRE(offsets_host[s + 1] >= offsets_host[s], "offsets must be non-decreasing");
  XT_REQUIRE(n_total < (1LL << 31), "at most 2^31 - 1 particles per call");
  XT_REQUIRE(n_total == 0 || xyzm, "NULL particle stream");
  XT_REQUIRE(((uintptr_t)xyzm & 15) == 0, "xyzm must be 16-byte aligned (float4 per particle)");
  const long long nchunk = bt_nchunk(offsets_host, nsnap);
  const BtLayout L = bt_layout(d, nsnap, n_total, nchunk, chunk);
  if (!workspace || workspace_bytes < L.total) {
    set_error("workspace of %zu bytes needed, %zu given", L.total, workspace_bytes);
    return XT_ERR_WORKSPACE;
  }
  const int nrow = (d.lmax + 1) * (d.lmax + 1);
  cudaStream_t st = as_stream(stream);
  char* ws = static_cast<char*>(workspace);
  float2* G = reinterpret_cast<float2*>(ws + L.G);
  int* ctr = reinterpret_cast<int*>(ws + L.ctr);      // [0] items, [1] item counter
  int* err = nullptr;
  XT_CUDA(cudaGetSymbolAddress((void**)&err, g_bt_err));
  XT_CUDA(cudaMemsetAsync(ctr, 0, 4 * sizeof(int), st));
  if (n_total == 0) {
    XT_CUDA(cudaMemsetAsync(G, 0, (size_t)nsnap * nrow * d.numr * sizeof(float2), st));
  } else {
    std::vector<BtChunk> chunks;
    std::vector<int> cfirst(nsnap + 1);
    chunks.reserve((size_t)nchunk);
    for (int s = 0; s < nsnap; ++s) {
      cfirst[s] = (int)chunks.size();
      for (long long b = offsets_host[s]; b < offsets_host[s + 1]; b += BT_SORT_CHUNK)
        chunks.push_back(BtChunk{s, 0, b, std::min(b + (long long)BT_SORT_CHUNK, offsets_host[s + 1])});
    }
    cfirst[nsnap] = (int)chunks.size();
    BtChunk* dchunks = reinterpret_cast<BtChunk*>(ws + L.chunks);
    int* dcfirst = reinterpret_cast<int*>(ws + L.cfirst);
    XT_CUDA(cudaMemcpyAsync(dchunks, chunks.data(), chunks.size() * sizeof(BtChunk), cudaMemcpyHostToDevice, st));
    XT_CUDA(cudaMemcpyAsync(dcfirst, cfirst.data(), cfirst.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    int* ccount = reinterpret_cast<int*>(ws + L.ccount);
    int* coff = reinterpret_cast<int*>(ws + L.coff);
    long long* bsize = reinterpret_cast<long long*>(ws + L.bsize);
    long long* bbase = reinterpret_cast<long long*>(ws + L.bbase);
    int* ifirst = reinterpret_cast<int*>(ws + L.ifirst);
    BtItem* items = reinterpret_cast<BtItem*>(ws + L.items);
    float4* sorted = reinterpret_cast<float4*>(ws + L.sorted);
    const float4* q = reinterpret_cast<const float4*>(xyzm);
    const int cgrid = (int)std::min<long long>(nchunk, (long long)sm_count() * 8);
    k_bt_hist<<<cgrid, 256, 0, st>>>(f, q, dchunks, (int)nchunk, L.nwin, ccount);
    XT_CHECK_LAUNCH("k_bt_hist");
    k_bt_offsets<<<nsnap, 256, 0, st>>>(dcfirst, L.nwin, ccount, coff, bsize);
    XT_CHECK_LAUNCH("k_bt_offsets");
    k_bt_buckets<<<1, 256, 0, st>>>(bsize, L.nb, chunk, bbase, ifirst, ctr);
    XT_CHECK_LAUNCH("k_bt_buckets");
    k_bt_items<<<(L.nb + 255) / 256, 256, 0, st>>>(bsize, bbase, ifirst, L.nb, L.nwin, chunk, items);
    XT_CHECK_LAUNCH("k_bt_items");
    k_bt_scatter<<<cgrid, 256, 0, st>>>(f, q, dchunks, (int)nchunk, L.nwin, coff, bbase, n_total, sorted,
                                        err);
    XT_CHECK_LAUNCH("k_bt_scatter");
    BtArgs A;
    A.T = f;
    A.sorted = sorted;
    A.items = items;
    A.nitems = ctr;
    A.counter = ctr + 1;
    A.partial = reinterpret_cast<float*>(ws + L.partial);
    A.err = err;
    A.nrow = nrow;
    A.no_odd = no_odd;
    int rc = with_lcap(d.lmax, [&](auto lc) -> int {
      constexpr int LC = decltype(lc)::value;
      constexpr int NPAD = ((LC + 1) * (LC + 1) + 15) / 16 * 16;
      return bt_with_stages<LC, NPAD>(stages, [&](auto sc) -> int {
        return bt_with_split(threads_per_particle, [&](auto pc) -> int {
          return bt_launch_gemm<LC, NPAD, decltype(sc)::value, decltype(pc)::value>(A, ctas_per_sm, st);
        });
      });
    });
    if (rc) return rc;
    const long long nred = (long long)nsnap * nrow;
    k_bt_reduce<<<(int)std::min<long long>(nred, (long long)sm_count() * 32), 256, 0, st>>>(
        A.partial, ifirst, d.fact, d.lmax, nsnap, nrow, d.numr, L.nwin, G);
    XT_CHECK_LAUNCH("k_bt_reduce");
  }
  const float2* efp_df = nullptr;
  XT_REQUIRE(sph_efp_df(handle, &efp_df), "NULL table handle");
  return launch_sph_contract_batched(efp_df, G, nsnap, d.lmax, d.nmax, d.numr, expcoef_out, st);
}

int xt_sph_batched_tc_residency(void* handle, int stages, int threads_per_particle, int* ctas_per_sm) {
  SphTab<double> d;
  XT_REQUIRE(sph_tabs(handle, &d, nullptr), "NULL table handle");
  XT_REQUIRE(stages >= 1 && stages <= 3, "stages must be 1, 2 or 3");
  XT_REQUIRE(threads_per_particle == 1 || threads_per_particle == 2, "threads_per_particle must be 1 or 2");
  XT_REQUIRE(ctas_per_sm, "NULL output");
  XT_REQUIRE(d.lmax <= 8, "the batched path supports lmax <= 8");
  int v = 0;
  with_lcap(d.lmax, [&](auto lc) -> int {
    constexpr int LC = decltype(lc)::value;
    constexpr int NPAD = ((LC + 1) * (LC + 1) + 15) / 16 * 16;
    return bt_with_stages<LC, NPAD>(stages, [&](auto sc) -> int {
      return bt_with_split(threads_per_particle, [&](auto pc) -> int {
        v = bt_residency<LC, NPAD, decltype(sc)::value, decltype(pc)::value>();
        return XT_OK;
      });
    });
  });
  *ctas_per_sm = v;
  XT_REQUIRE(v >= 1, "k_sph_batched_tc does not fit on an SM at %d stages", stages);
  return XT_OK;
}

int xt_sph_batched_tc_status(void) {
  int* err = nullptr;
  XT_CUDA(cudaDeviceSynchronize());
  XT_CUDA(cudaGetSymbolAddress((void**)&err, g_bt_err));
  int v = 0;
  XT_CUDA(cudaMemcpy(&v, err, sizeof(int), cudaMemcpyDeviceToHost));
  if (v) {
    const int zero = 0;
    XT_CUDA(cudaMemcpy(err, &zero, sizeof(int), cudaMemcpyHostToDevice));
    set_error("batched tensor-core accumulation: %s", v == 1 ? "an MMA wait timed out"
                                                            : (v == 2 ? "a sorted slot fell outside its bucket"
                                                                      : "a particle fell outside its window"));
    return XT_ERR_DEVICE;
  }
  return XT_OK;
}

}  // extern "C"
