// Learned radial basis, pass 1 on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory).
//
// Same mathematics as k_mlp_radial (xt_mlp_eval.cu): for every point and
// network l, silu layers 2 and 3 and the coefficient-folded last layer, with
// BF16 operands and FP32 accumulation.  Organisation:
//   * one CTA per SM (the shared-memory footprint keeps a second CTA out, so
//     the tensor-memory allocation never waits), each on one network l and a
//     contiguous range of tiles;
//   * two warpgroups per CTA, each with its own 128-point tile (one point per
//     TMEM lane / thread), activation buffer, tensor-memory columns and
//     mbarrier: while one warpgroup runs its epilogue the tensor core works
//     on the other's layer;
//   * weights of the current network sit in shared memory in the canonical
//     K-major, no-swizzle layout (8-row x 16-byte core matrices; 128 B between
//     core matrices along K, 2048 B between 8-row groups);
//   * the activation tile A (128 x 128 BF16) is rebuilt in the same layout by
//     the epilogue of every layer: tcgen05.ld of the thread's accumulator row,
//     bias, SiLU, BF16 packing, 16-byte shared stores;
//   * one elected thread issues the MMAs (M = 128, N = 128 or 32, K = 16 per
//     instruction) and commits them to an mbarrier; waits are bounded and a
//     timeout sets an error flag, frees the tensor memory and returns.
#include <cmath>

#include "xt_mlp.cuh"
#include "xt_tc.cuh"

namespace xt {

constexpr int TC_M = 128;
constexpr int TC_HID = MLP_HID;
constexpr int TC_NC = MLP_NC;
constexpr int TC_LBO = 128;                       // bytes between core matrices along K
constexpr int TC_SBO = (TC_HID / 8) * 128;        // bytes between 8-row groups (K = 128)
constexpr int TC_WG = 4;                          // warpgroups per CTA, each owning one tile in flight
constexpr int TC_THREADS = 128 * TC_WG;
constexpr int TC_TMEM_COLS = 512;                 // warpgroup g: columns [128g, 128g+128); the last layer
                                                  // reuses the first 32 once layer 3 has been read out

// shared-memory map (bytes)
constexpr int TC_OFF_W2 = 0;
constexpr int TC_OFF_W3 = TC_OFF_W2 + TC_HID * TC_HID * 2;        // 32 KB each
constexpr int TC_OFF_W4H = TC_OFF_W3 + TC_HID * TC_HID * 2;
constexpr int TC_OFF_W4L = TC_OFF_W4H + TC_NC * TC_HID * 2;       // 8 KB each
constexpr int TC_OFF_A = TC_OFF_W4L + TC_NC * TC_HID * 2;         // TC_WG activation tiles of 32 KB
constexpr int TC_A_BYTES = TC_M * TC_HID * 2;
constexpr int TC_OFF_F = TC_OFF_A + TC_WG * TC_A_BYTES;          // w1 b1 b2 b3 [128] b4 [32] floats
constexpr int TC_OFF_CS = TC_OFF_F + (4 * TC_HID + TC_NC) * 4;    // prior weights of this l [15][32], 1/n [32]
constexpr int TC_CS_ROWS = 2 * MLP_LMAX + 1;
constexpr int TC_OFF_BAR = TC_OFF_CS + (TC_CS_ROWS * MLP_KMAX + MLP_KMAX) * 4;   // mbarriers, tmem slot, fail flags
constexpr int TC_SMEM = TC_OFF_BAR + 64;
static_assert(TC_OFF_A % 1024 == 0 && TC_A_BYTES % 1024 == 0 && TC_OFF_BAR % 8 == 0, "alignment");
static_assert(2 * TC_SMEM > 228 * 1024, "one CTA per SM keeps the tensor-memory allocation uncontended");
static_assert(TC_SMEM <= 227 * 1024, "dynamic shared memory per CTA");

// Byte offset of element (row, k) of a K-major canonical tile with K = 128.
__device__ __forceinline__ int tc_off(int row, int k) {
  return (row >> 3) * TC_SBO + (k >> 3) * TC_LBO + (row & 7) * 16 + (k & 7) * 2;
}

// Stage weights [rows][128] (row-major BF16, global) into a canonical tile.
__device__ __forceinline__ void tc_stage(unsigned char* dst, const __nv_bfloat16* src, int rows) {
  for (int c = threadIdx.x; c < rows * (TC_HID / 8); c += blockDim.x) {
    const int row = c / (TC_HID / 8), k8 = c % (TC_HID / 8);
    *reinterpret_cast<uint4*>(dst + tc_off(row, k8 * 8)) =
        *reinterpret_cast<const uint4*>(src + (size_t)row * TC_HID + k8 * 8);
  }
}

// Epilogue of a hidden layer for this thread's row: A[row][:] = bf16(silu(acc + b))
// with hb = b / 2.
__device__ __forceinline__ void tc_hidden_epilogue(uint32_t tmem_row, const float* hb, unsigned char* A, int row) {
#pragma unroll 1
  for (int c = 0; c < TC_HID / 32; ++c) {
    float v[32];
    tc_ld32(tmem_row + 32 * c, v);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const float4 b0 = *reinterpret_cast<const float4*>(hb + 32 * c + 8 * q);
      const float4 b1 = *reinterpret_cast<const float4*>(hb + 32 * c + 8 * q + 4);
      const float* w = v + 8 * q;
      const uint32_t p0 = pack_bf16x2(silu_h(fmaf(w[0], 0.5f, b0.x)), silu_h(fmaf(w[1], 0.5f, b0.y)));
      const uint32_t p1 = pack_bf16x2(silu_h(fmaf(w[2], 0.5f, b0.z)), silu_h(fmaf(w[3], 0.5f, b0.w)));
      const uint32_t p2 = pack_bf16x2(silu_h(fmaf(w[4], 0.5f, b1.x)), silu_h(fmaf(w[5], 0.5f, b1.y)));
      const uint32_t p3 = pack_bf16x2(silu_h(fmaf(w[6], 0.5f, b1.z)), silu_h(fmaf(w[7], 0.5f, b1.w)));
      *reinterpret_cast<uint4*>(A + tc_off(row, 32 * c + 8 * q)) = make_uint4(p0, p1, p2, p3);
    }
  }
}

__device__ __forceinline__ int tc_band(float lr, float lnr0, float inv_bw, int nb) {
  int b = (int)((lr - lnr0) * inv_bw);
  return b < 0 ? 0 : (b >= nb ? nb - 1 : b);
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_mlp_radial_tc(TcArgs a, int ctas_per_net) {
  extern __shared__ __align__(1024) unsigned char sm[];
  unsigned char* W2s = sm + TC_OFF_W2;
  unsigned char* W3s = sm + TC_OFF_W3;
  unsigned char* W4h = sm + TC_OFF_W4H;
  unsigned char* W4l = sm + TC_OFF_W4L;
  float* w1 = reinterpret_cast<float*>(sm + TC_OFF_F);
  float* b1 = w1 + TC_HID;
  float* b2 = b1 + TC_HID;
  float* b3 = b2 + TC_HID;
  float* b4 = b3 + TC_HID;
  float* cs = reinterpret_cast<float*>(sm + TC_OFF_CS);        // [rr][n], rows l^2 + rr
  float* inv_n = cs + TC_CS_ROWS * MLP_KMAX;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + TC_OFF_BAR);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + TC_OFF_BAR + 8 * TC_WG);
  int* fails = reinterpret_cast<int*>(sm + TC_OFF_BAR + 8 * TC_WG + 4);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int g = warp >> 2, wtid = tid & 127, bar_id = 1 + g;
  const int l = blockIdx.x / ctas_per_net, chunk = blockIdx.x % ctas_per_net;
  unsigned char* A = sm + TC_OFF_A + g * TC_A_BYTES;
  const uint32_t bar_g = smem_u32(bars + g);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid < TC_WG) {
    mbar_init(smem_u32(bars + tid));
    fails[tid] = 0;
  }
  // network l: weights in the canonical layout, first-layer and bias vectors
  {
    const __nv_bfloat16* gw = a.wb + (size_t)l * a.psize;
    const float* gp = a.params + (size_t)l * a.psize;
    tc_stage(W2s, gw + MlpLayout::W2, TC_HID);
    tc_stage(W3s, gw + MlpLayout::W3, TC_HID);
    tc_stage(W4h, a.w4h + (size_t)l * TC_NC * TC_HID, TC_NC);
    tc_stage(W4l, a.w4l + (size_t)l * TC_NC * TC_HID, TC_NC);
    for (int i = tid; i < TC_HID; i += blockDim.x) {      // halved: silu(z) = silu_h(z / 2)
      w1[i] = 0.5f * gp[MlpLayout::W1 + i];
      b1[i] = 0.5f * gp[MlpLayout::B1 + i];
      b2[i] = 0.5f * gp[MlpLayout::B2 + i];
      b3[i] = 0.5f * gp[MlpLayout::B3 + i];
    }
    for (int i = tid; i < TC_NC; i += blockDim.x) b4[i] = a.b4c[l * TC_NC + i];
    if (a.CS)
      for (int i = tid; i < (2 * l + 1) * a.K; i += blockDim.x)
        cs[(i / a.K) * MLP_KMAX + i % a.K] = a.CS[(size_t)(l * l) * a.K + i];
    for (int i = tid; i < MLP_KMAX; i += blockDim.x) inv_n[i] = i ? 1.f / (float)i : 0.f;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_g = *tmem_slot + 128u * g;
  const uint32_t tmem_row = tmem_g + ((uint32_t)(32 * (warp & 3)) << 16);   // this warp's 32 lanes
  const uint32_t idesc_h = tc_idesc(TC_M, TC_HID), idesc_o = tc_idesc(TC_M, TC_NC);
  const int nout = 2 * (2 * l + 1);
  uint32_t phase = 0;
  bool ok = true;

  const long long ntile = (a.n + TC_M - 1) / TC_M;
  const long long t0 = ntile * chunk / ctas_per_net, t1 = ntile * (chunk + 1) / ctas_per_net;
  // the next tile's point is loaded one tile ahead
  float4 nxt = make_float4(1.f, 0.f, 0.f, 0.f);
  if (t0 + g < t1 && (t0 + g) * TC_M + wtid < a.n) nxt = a.xyzw[(t0 + g) * TC_M + wtid];
  for (long long tile = t0 + g; tile < t1 && ok; tile += TC_WG) {
    const long long p = tile * TC_M + wtid;
    const bool valid = p < a.n;
    const float4 v = nxt;
    const long long pn = p + (long long)TC_WG * TC_M;
    if (tile + TC_WG < t1 && pn < a.n) nxt = a.xyzw[pn];
    float r = 1.f;
    if (valid) r = sqrtf(fmaf(v.x, v.x, fmaf(v.y, v.y, v.z * v.z)));
    r = fminf(fmaxf(r, a.rmin), a.rmax);
    const float lr = logf(r);
    const bool use = valid && a.band_use[tc_band(lr, a.lnr0, a.inv_bw, a.nb)] != 0;
    if (!wg_any(use, bar_id)) continue;
    // layer 1 into this warpgroup's activation tile (w1, b1 halved)
    const float t = fminf(fmaxf((lr - a.c0) * a.c1, -1.f), 1.f);
#pragma unroll 1
    for (int c = 0; c < TC_HID / 8; ++c) {
      const float4 wa = *reinterpret_cast<const float4*>(w1 + 8 * c), wb = *reinterpret_cast<const float4*>(w1 + 8 * c + 4);
      const float4 ba = *reinterpret_cast<const float4*>(b1 + 8 * c), bb = *reinterpret_cast<const float4*>(b1 + 8 * c + 4);
      const uint32_t p0 = pack_bf16x2(silu_h(fmaf(t, wa.x, ba.x)), silu_h(fmaf(t, wa.y, ba.y)));
      const uint32_t p1 = pack_bf16x2(silu_h(fmaf(t, wa.z, ba.z)), silu_h(fmaf(t, wa.w, ba.w)));
      const uint32_t p2 = pack_bf16x2(silu_h(fmaf(t, wb.x, bb.x)), silu_h(fmaf(t, wb.y, bb.y)));
      const uint32_t p3 = pack_bf16x2(silu_h(fmaf(t, wb.z, bb.z)), silu_h(fmaf(t, wb.w, bb.w)));
      *reinterpret_cast<uint4*>(A + tc_off(wtid, 8 * c)) = make_uint4(p0, p1, p2, p3);
    }
    // layers 2, 3 (hidden) and 4 (folded, hi + lo)
#pragma unroll 1
    for (int layer = 0; layer < 3; ++layer) {
      fence_async_smem();
      tc_fence_before();
      wg_sync(bar_id);
      tc_fence_after();
      if (wtid == 0) {
        const uint32_t a_base = smem_u32(A);
        if (layer < 2) {
          const uint32_t w_base = smem_u32(layer == 0 ? W2s : W3s);
#pragma unroll
          for (int k = 0; k < TC_HID / 16; ++k)
            tc_mma(tmem_g, tc_desc(a_base + k * 2 * TC_LBO, TC_LBO, TC_SBO),
                   tc_desc(w_base + k * 2 * TC_LBO, TC_LBO, TC_SBO), idesc_h, k > 0);
        } else {
          const uint32_t h_base = smem_u32(W4h), l_base = smem_u32(W4l);
#pragma unroll
          for (int k = 0; k < TC_HID / 16; ++k)
            tc_mma(tmem_g, tc_desc(a_base + k * 2 * TC_LBO, TC_LBO, TC_SBO),
                   tc_desc(h_base + k * 2 * TC_LBO, TC_LBO, TC_SBO), idesc_o, k > 0);
#pragma unroll
          for (int k = 0; k < TC_HID / 16; ++k)
            tc_mma(tmem_g, tc_desc(a_base + k * 2 * TC_LBO, TC_LBO, TC_SBO),
                   tc_desc(l_base + k * 2 * TC_LBO, TC_LBO, TC_SBO), idesc_o, 1);
        }
        tc_commit(bar_g);
      }
      if (!mbar_wait(bar_g, phase)) fails[g] = 1;
      wg_sync(bar_id);
      if (fails[g]) {
        // the commit may still be outstanding: one more bounded wait before
        // the tensor memory is released
        mbar_wait(bar_g, phase);
        ok = false;
        break;
      }
      phase ^= 1;
      tc_fence_after();
      if (layer < 2) {
        tc_hidden_epilogue(tmem_row, layer == 0 ? b2 : b3, A, wtid);
      } else {
        // folded network sums + bias; with a.CS set, also the prior (the
        // R row is then the full radial sums per coefficient row).  Measured
        // on GB300 the prior is cheaper in the second pass, which runs at
        // higher occupancy, so the evaluation leaves a.CS unset.
        float v[32];
        tc_ld32(tmem_row, v);
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] += b4[i];
        const float u = r * a.a_inv;
        if (a.CS) ho_radial<float>(u, l, a.K, inv_n, [&](int n, float ho, float uho) {
#pragma unroll
          for (int rr = 0; rr < TC_CS_ROWS; ++rr) {
            if (rr <= 2 * l) {
              const float c = cs[rr * MLP_KMAX + n];
              v[2 * rr] = fmaf(c, ho, v[2 * rr]);
              v[2 * rr + 1] = fmaf(c, uho, v[2 * rr + 1]);
            }
          }
        });
        if (use) {
          float* dst = a.R + p * a.rstride + 2 * l * l;
#pragma unroll
          for (int i = 0; i < 32; i += 2)
            if (i < nout) *reinterpret_cast<float2*>(dst + i) = make_float2(v[i], v[i + 1]);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (tid < TC_WG && fails[tid]) atomicExch(a.err, 1);
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(*tmem_slot), "r"(TC_TMEM_COLS)
                 : "memory");
  }
}

static __device__ int g_tc_err;

int tc_error_flag(int** dptr) {
  XT_CUDA(cudaGetSymbolAddress((void**)dptr, g_tc_err));
  return XT_OK;
}

// Host launcher, called by xt_learned_eval and xt_learned_radial_pass.
int launch_mlp_radial_tc(const TcArgs& a, int nsm, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    XT_CUDA(cudaFuncSetAttribute(k_mlp_radial_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
    attr = true;
  }
  // one CTA per SM, an equal number per network
  int per = nsm / a.L;
  if (per < 1) per = 1;
  k_mlp_radial_tc<<<(unsigned)(per * a.L), TC_THREADS, TC_SMEM, st>>>(a, per);
  XT_CHECK_LAUNCH("k_mlp_radial_tc");
  return XT_OK;
}

}  // namespace xt
