// Learned radial basis, part 1: training of the per-l networks on the GPU.
//
// All products run on the tensor cores as BF16 x BF16 -> FP32 (mma.sync
// m16n8k16): weights are FP32 masters updated by Adam with BF16 copies for
// the products, activations are stored in BF16 after the FP32 epilogue.  The
// L networks (one per harmonic l) are batched along grid.z.  Labels come from
// the method's own SL tables (table interpolation of phi_nl and dphi_nl/dr,
// the functions the table path evaluates) minus the analytic prior.
#include <cmath>
#include <cstring>
#include <vector>

#include "xt_mlp.cuh"
#include "xt_tc.cuh"

namespace xt {

constexpr int HID = MLP_HID;
constexpr int NOP = MLP_NOP;

// ------------------------------------------------------------------ tensor-core GEMM
// C[M x N] = opA(A) [M x K] * opB(B) [K x N], BF16 operands, FP32 accumulation.
//   TA = 0: A stored [M][lda] (k contiguous);  TA = 1: A stored [K][lda] (m contiguous)
//   TB = 0: B stored [N][ldb] (k contiguous);  TB = 1: B stored [K][ldb] (n contiguous)
// blockIdx.z = l * ksplit + kpart (the L networks batched along z, split-K
// parts accumulated by EPI_ATOMIC).
enum { EPI_STORE = 0, EPI_BIAS_SILU = 1, EPI_DSILU = 2, EPI_ATOMIC = 3, EPI_BIAS = 4 };

struct GemmArgs {
  const __nv_bfloat16* A;
  const __nv_bfloat16* B;
  int M, N, K, lda, ldb;
  long long sA, sB;          // per-network strides (elements)
  int ksplit;
  float* C;                  // fp32 output / accumulation target
  int ldc;
  long long sC;
  const float* bias;         // per-network bias (EPI_BIAS*), stride sBias
  long long sBias;
  __nv_bfloat16* Hout;       // bf16 activation output (EPI_BIAS_SILU, EPI_DSILU), ld = ldc, stride sC
  const float* Zsaved;       // pre-activations for EPI_DSILU (ld = ldc, stride sC)
  int* err;                  // set to 1 on an MMA wait timeout (the learned path's flag, xt_learned_status)
};

// One CTA per 128 x BN output tile on the 5th-generation tensor cores: K in
// steps of 64, both operands staged by cp.async (16-byte copies, rows beyond M
// zero-filled) into the canonical no-swizzle layouts, K-major when the
// operand is stored k-contiguous (8-row x 16-byte core matrices, 128 bytes
// apart along K, 1024 apart across 8-row groups) and MN-major when it is
// stored m- or n-contiguous (8 x 16-byte core matrices along the rows, 128
// bytes apart, k groups of 8 a full tile width apart; instruction-descriptor
// bits 15 and 16); two stages, so the copies of step k+1 run while the MMAs
// of step k do.  One thread issues the four K = 16 MMAs of a step and commits
// them to the stage's mbarrier; waits are bounded and a timeout sets the
// learned path's error flag (read by xt_learned_status).  The FP32 accumulator (128 lanes x BN columns of tensor
// memory) is read by tcgen05.ld for the epilogue and transposed through
// shared memory, so that the stores (and the bias, Z and atomic accesses) are
// row segments of 32 consecutive columns per warp instruction.
constexpr int GT_M = 128, GT_BK = 64, GT_STAGES = 2;

template <int BN>
struct GtTile {
  static constexpr int A_BYTES = GT_M * GT_BK * 2;
  static constexpr int B_BYTES = BN * GT_BK * 2;
  static constexpr int STAGE = A_BYTES + B_BYTES;
  static constexpr int SMEM = GT_STAGES * STAGE + 64;
};

__device__ __forceinline__ void cp16(uint32_t dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Copies of one operand tile (ROWS x 64 of K) into the canonical layout.
template <int T, int ROWS>
__device__ __forceinline__ void gt_stage(uint32_t dst, const __nv_bfloat16* src, int ld, int r0, int rmax, int k0) {
  if (T == 0) {                                   // [rows][ld], k contiguous: K-major
    for (int c = threadIdx.x; c < ROWS * (GT_BK / 8); c += blockDim.x) {
      const int row = c >> 3, kc = c & 7;
      const bool ok = r0 + row < rmax;
      cp16(dst + (row >> 3) * ((GT_BK / 8) * 128) + kc * 128 + (row & 7) * 16,
           ok ? src + (size_t)(r0 + row) * ld + k0 + 8 * kc : src, ok);
    }
  } else {                                        // [k][ld], rows contiguous: MN-major
    for (int c = threadIdx.x; c < GT_BK * (ROWS / 8); c += blockDim.x) {
      const int k = c / (ROWS / 8), rc = c % (ROWS / 8);
      const bool ok = r0 + 8 * rc < rmax;
      cp16(dst + (k >> 3) * ((ROWS / 8) * 128) + rc * 128 + (k & 7) * 16,
           ok ? src + (size_t)(k0 + k) * ld + r0 + 8 * rc : src, ok);
    }
  }
}

template <int T, int ROWS>
__device__ __forceinline__ uint64_t gt_desc(uint32_t base, int kk) {
  if (T == 0) return tc_desc(base + kk * 256, 128, (GT_BK / 8) * 128);
  return tc_desc(base + kk * 2 * ((ROWS / 8) * 128), (ROWS / 8) * 128, 128);
}

template <int TA, int TB, int EPI, int BN>
__global__ void __launch_bounds__(128) k_gemm_tc(GemmArgs g) {
  using TL = GtTile<BN>;
  extern __shared__ __align__(1024) unsigned char sm[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + GT_STAGES * TL::STAGE);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + GT_STAGES);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int l = blockIdx.z / g.ksplit, kpart = blockIdx.z % g.ksplit;
  const __nv_bfloat16* A = g.A + l * g.sA;
  const __nv_bfloat16* B = g.B + l * g.sB;
  const int m0 = blockIdx.x * GT_M, n0 = blockIdx.y * BN;
  const int kchunk = g.K / g.ksplit, kbeg = kpart * kchunk;
  const int nk = kchunk / GT_BK;
  constexpr int NCOLS = BN < 32 ? 32 : BN;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid < GT_STAGES) mbar_init(smem_u32(bars + tid));
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc_idesc(GT_M, BN) | ((uint32_t)TA << 15) | ((uint32_t)TB << 16);
  const uint32_t s0 = smem_u32(sm);
  auto load = [&](int step) {
    const uint32_t st = s0 + (step % GT_STAGES) * TL::STAGE;
    const int k0 = kbeg + step * GT_BK;
    gt_stage<TA, GT_M>(st, A, g.lda, m0, g.M, k0);
    gt_stage<TB, BN>(st + TL::A_BYTES, B, g.ldb, n0, g.N, k0);
  };
  bool ok = true;
  load(0);
  cp_commit();
  for (int ks = 0; ks < nk; ++ks) {
    if (ks + 1 < nk) {
      // the next stage's buffer was last read by the MMAs of step ks - 1
      bool lf = false;
      if (ks >= 1 && tid == 0)
        lf = !mbar_wait(smem_u32(bars + (ks - 1) % GT_STAGES), (uint32_t)(((ks - 1) / GT_STAGES) & 1));
      if (__syncthreads_or(lf)) {
        ok = false;
        break;
      }
      load(ks + 1);
    }
    cp_commit();
    cp_wait1();                                   // this thread's copies of step ks have landed
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
      const uint32_t st = s0 + (ks % GT_STAGES) * TL::STAGE;
#pragma unroll
      for (int kk = 0; kk < GT_BK / 16; ++kk)
        tc_mma(tmem, gt_desc<TA, GT_M>(st, kk), gt_desc<TB, BN>(st + TL::A_BYTES, kk), idesc,
               (ks > 0 || kk > 0) ? 1u : 0u);
      tc_commit(smem_u32(bars + ks % GT_STAGES));
    }
  }
  if (ok && nk > 0) {
    bool lf = false;
    if (tid == 0) lf = !mbar_wait(smem_u32(bars + (nk - 1) % GT_STAGES), (uint32_t)(((nk - 1) / GT_STAGES) & 1));
    if (__syncthreads_or(lf)) ok = false;
  }
  if (ok) {
    tc_fence_after();
    asm volatile("cp.async.wait_all;" ::: "memory");   // no copy in flight into the reused stage memory
    __syncthreads();
    float* C = g.C + l * g.sC;
    const float* bias = g.bias ? g.bias + l * g.sBias : nullptr;
    __nv_bfloat16* H = g.Hout ? g.Hout + l * g.sC : nullptr;
    const float* Z = g.Zsaved ? g.Zsaved + l * g.sC : nullptr;
    // each warp's 32 rows x 32 columns pass through shared memory (the
    // stage buffers, free now) so that every global access below is one
    // contiguous row segment per warp instruction
    float* T = reinterpret_cast<float*>(sm) + warp * (32 * 33);
    const int lane = tid & 31;
    const int mw = m0 + 32 * warp;
#pragma unroll 1
    for (int c = 0; c < BN / 32; ++c) {
      float v[32];
      tc_ld32(tmem + ((uint32_t)(32 * warp) << 16) + 32 * c, v);   // row mw + lane, all lanes (.sync.aligned)
#pragma unroll
      for (int i = 0; i < 32; ++i) T[lane * 33 + i] = v[i];
      __syncwarp();
      const int n = n0 + 32 * c + lane;
      const float b = (EPI == EPI_BIAS || EPI == EPI_BIAS_SILU) ? bias[n] : 0.f;
      const int rows = nk > 0 ? min(32, g.M - mw) : 0;
      // the saved pre-activations of the 32 rows, all in flight at once
      float zv[32];
      if (EPI == EPI_DSILU) {
#pragma unroll
        for (int r = 0; r < 32; ++r) zv[r] = r < rows ? Z[(size_t)(mw + r) * g.ldc + n] : 0.f;
      }
#pragma unroll
      for (int r = 0; r < 32; ++r) {
        if (r >= rows) break;
        const size_t idx = (size_t)(mw + r) * g.ldc + n;
        float q = T[r * 33 + lane];
        if (EPI == EPI_ATOMIC) {
          atomicAdd(C + idx, q);
          continue;
        }
        q += b;
        if (EPI == EPI_DSILU) q *= dsilu_fast(zv[r]);
        C[idx] = q;                          // pre-activation (SILU) / dZ in FP32 (DSILU)
        if (EPI == EPI_BIAS_SILU) H[idx] = __float2bfloat16_rn(silu_fast(q));
        else if (EPI == EPI_DSILU) H[idx] = __float2bfloat16_rn(q);
      }
      __syncwarp();
    }
  } else if (tid == 0) {
    atomicExch(g.err, 1);
    // MMAs possibly in flight finish (bounded) before the tensor memory is released
    if (nk > 0) mbar_wait(smem_u32(bars + (nk - 1) % GT_STAGES), (uint32_t)(((nk - 1) / GT_STAGES) & 1));
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOLS) : "memory");
  }
}

// ------------------------------------------------------------------ small kernels
// layer 1 forward: Z1[b][j] = t_b W1[j] + b1[j], H1 = bf16(silu(Z1))
__global__ void k_mlp_l1_fwd(const float* __restrict__ params, int psize, const float* __restrict__ t, int B,
                             float* __restrict__ Z1, __nv_bfloat16* __restrict__ H1) {
  const int l = blockIdx.y;
  const float* p = params + (size_t)l * psize;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < B * HID; idx += gridDim.x * blockDim.x) {
    const int b = idx / HID, j = idx % HID;
    const float z = fmaf(t[b], p[MlpLayout::W1 + j], p[MlpLayout::B1 + j]);
    Z1[(size_t)l * B * HID + idx] = z;
    H1[(size_t)l * B * HID + idx] = __float2bfloat16_rn(silu_fast(z));
  }
}

template <int NT>
__device__ __forceinline__ float block_sum(float v, float* sh) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  float a = 0.f;
  if (threadIdx.x == 0)
    for (int w = 0; w < NT / 32; ++w) a += sh[w];
  return a;
}

// layer 1 backward: dW1[j] = sum_b dZ1[b][j] t_b, db1[j] = sum_b dZ1[b][j]; block per (j, l)
__global__ void __launch_bounds__(256) k_mlp_l1_bwd(const float* __restrict__ dZ1, const float* __restrict__ t,
                                                    int B, float* __restrict__ grads, int psize) {
  const int l = blockIdx.y, j = blockIdx.x;
  const float* d = dZ1 + (size_t)l * B * HID;
  float sw = 0.f, sb = 0.f;
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    const float v = d[(size_t)b * HID + j];
    sw = fmaf(v, t[b], sw);
    sb += v;
  }
  __shared__ float s1[8], s2[8];
  const float a = block_sum<256>(sw, s1);
  const float c = block_sum<256>(sb, s2);
  if (threadIdx.x == 0) {
    grads[(size_t)l * psize + MlpLayout::W1 + j] = a;
    grads[(size_t)l * psize + MlpLayout::B1 + j] = c;
  }
}

// bias gradient: grads[boff + j] = sum_b dZ[b][j], j < ncol (ld = ldz); block per (j, l)
__global__ void __launch_bounds__(256) k_mlp_bias_grad(const float* __restrict__ dZ, int B, int ldz, int ncol,
                                                       float* __restrict__ grads, int psize, int boff) {
  const int l = blockIdx.y, j = blockIdx.x;
  if (j >= ncol) return;
  const float* d = dZ + (size_t)l * B * ldz;
  float s = 0.f;
  for (int b = threadIdx.x; b < B; b += blockDim.x) s += d[(size_t)b * ldz + j];
  __shared__ float sh[8];
  const float a = block_sum<256>(s, sh);
  if (threadIdx.x == 0) grads[(size_t)l * psize + boff + j] = a;
}

// MSE over the nout real outputs: dY = 2 (Y - T) / (B nout) (zero on padding
// columns), its BF16 copy, and the FP64 loss per network.  T: per-network
// stride ldT, row pitch NOP.
__global__ void k_mlp_loss(const float* __restrict__ Y, const float* __restrict__ T, long long ldT, int B, int nout,
                           float* __restrict__ dY, __nv_bfloat16* __restrict__ dYb, double* __restrict__ loss) {
  const int l = blockIdx.y;
  double local = 0.0;
  const float inv = 2.f / ((float)B * nout);
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < B * NOP; idx += gridDim.x * blockDim.x) {
    const int o = idx % NOP;
    const size_t k = (size_t)l * B * NOP + idx;
    float d = 0.f;
    if (o < nout) {
      const float r = Y[k] - T[(size_t)l * ldT + idx];
      local += (double)r * r;
      d = r * inv;
    }
    dY[k] = d;
    dYb[k] = __float2bfloat16_rn(d);
  }
  for (int off = 16; off > 0; off >>= 1) local += __shfl_down_sync(0xffffffffu, local, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss + l, local / ((double)B * nout));
}

__device__ __forceinline__ bool padded_output(int o, int nout) {
  if (o >= MlpLayout::W4 && o < MlpLayout::B4) return (o - MlpLayout::W4) / HID >= nout;
  if (o >= MlpLayout::B4) return (o - MlpLayout::B4) >= nout;
  return false;
}

// Adam (Kingma & Ba 2015) on the FP32 masters; refreshes the BF16 copies.
// Output rows >= nout stay zero.
__global__ void k_mlp_adam(float* __restrict__ params, const float* __restrict__ grads, float* __restrict__ m1,
                           float* __restrict__ m2, __nv_bfloat16* __restrict__ wb, int total, int psize, int nout,
                           float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int o = i % psize;
    if (padded_output(o, nout)) {
      params[i] = 0.f;
      wb[i] = __float2bfloat16_rn(0.f);
      continue;
    }
    const float gr = grads[i];
    const float a = b1 * m1[i] + (1.f - b1) * gr;
    const float v = b2 * m2[i] + (1.f - b2) * gr * gr;
    m1[i] = a;
    m2[i] = v;
    const float w = params[i] - lr * (a / c1) / (sqrtf(v / c2) + eps);
    params[i] = w;
    wb[i] = __float2bfloat16_rn(w);
  }
}

__global__ void k_mlp_refresh(float* __restrict__ params, __nv_bfloat16* __restrict__ wb, int total, int psize,
                              int nout) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    if (padded_output(i % psize, nout)) params[i] = 0.f;
    wb[i] = __float2bfloat16_rn(params[i]);
  }
}

// ------------------------------------------------------------------ labels
// Training targets from the SL tables.  For radius r (clamped to the table
// range, as the table interpolation clamps), for l <= lmax and n < K:
//   T[l][p][n]   = (phi_nl(r) - s_nl HO_nl(r/a)) / sig[l][n]
//   T[l][p][K+n] = (r dphi_nl/dr - s_nl u dHO_nl/du) / sig[l][K+n]
// with phi_nl and dphi_nl/dr the table interpolation of spheresl
// get_halo_dens_pot_force (spheresl.py:106-160): the pot-like lerp product
// and the 3-point force stencil.  t[p] is the network input.
__global__ void __launch_bounds__(128) k_mlp_labels(SphTab<double> T, const double* __restrict__ efp, int K,
                                                    const double* __restrict__ r, long long n, double a_prior,
                                                    const double* __restrict__ s, const double* __restrict__ sig,
                                                    double rmin, double rmax, double c0, double c1,
                                                    float* __restrict__ t_out, float* __restrict__ T_out,
                                                    long long ldT) {
  __shared__ double inv_n[MLP_KMAX];
  if (threadIdx.x < MLP_KMAX) inv_n[threadIdx.x] = threadIdx.x ? 1.0 / threadIdx.x : 0.0;
  __syncthreads();
  const int nmax = T.nmax, numr = T.numr;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const double rp = r[p];
    const double rc = fmin(fmax(rp, rmin), rmax);
    double tv = (log(rc) - c0) * c1;
    tv = fmin(fmax(tv, -1.0), 1.0);
    t_out[p] = (float)tv;
    const SphBins<double> B = sph_bins(T, rc, true, false);
    for (int l = 0; l <= T.lmax; ++l) {
      float* out = T_out + (size_t)l * ldT + (size_t)p * NOP;
      const double* sl = s + l * K;
      const double* gl = sig + l * 2 * K;
      ho_radial<double>(rc / a_prior, l, K, inv_n, [&](int k, double ho, double uho) {
        const double* g = efp + ((size_t)l * nmax + k) * numr + (B.j - 1);
        const double phi = B.wp[0] * g[0] + B.wp[1] * g[1] + B.wp[2] * g[2];
        const double dphi = B.wf[0] * g[0] + B.wf[1] * g[1] + B.wf[2] * g[2];
        out[k] = (float)((phi - sl[k] * ho) / gl[k]);
        out[K + k] = (float)((rc * dphi - sl[k] * uho) / gl[K + k]);
      });
      for (int o = 2 * K; o < NOP; ++o) out[o] = 0.f;
    }
  }
}

// ------------------------------------------------------------------ workspace
static size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

struct MlpWork {
  float *Z1, *Z2, *Z3, *Y, *dY, *dZ3, *dZ2, *dZ1;
  __nv_bfloat16 *H1, *H2, *H3, *dYb, *dZ3b, *dZ2b;
  double* loss;
  size_t total;
};

static MlpWork mlp_work(void* ws, int L, int B) {
  MlpWork w{};
  char* base = static_cast<char*>(ws);
  size_t o = 0;
  auto takef = [&](size_t n) {
    float* p = reinterpret_cast<float*>(base ? base + o : nullptr);
    o += al(n * 4);
    return p;
  };
  auto takeb = [&](size_t n) {
    __nv_bfloat16* p = reinterpret_cast<__nv_bfloat16*>(base ? base + o : nullptr);
    o += al(n * 2);
    return p;
  };
  const size_t lh = (size_t)L * B * HID, lo = (size_t)L * B * NOP;
  w.Z1 = takef(lh); w.Z2 = takef(lh); w.Z3 = takef(lh); w.Y = takef(lo); w.dY = takef(lo);
  w.dZ3 = takef(lh); w.dZ2 = takef(lh); w.dZ1 = takef(lh);
  w.H1 = takeb(lh); w.H2 = takeb(lh); w.H3 = takeb(lh); w.dYb = takeb(lo); w.dZ3b = takeb(lh); w.dZ2b = takeb(lh);
  w.loss = reinterpret_cast<double*>(base ? base + o : nullptr);
  o += al((size_t)L * 8);
  w.total = o;
  return w;
}

template <int TA, int TB, int EPI, int BN>
static int gemm_bn(const GemmArgs& a, int L, cudaStream_t st) {
  auto kern = k_gemm_tc<TA, TB, EPI, BN>;
  static bool attr = false;
  if (!attr) {
    XT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, GtTile<BN>::SMEM));
    attr = true;
  }
  GemmArgs b = a;
  int rc = tc_error_flag(&b.err);
  if (rc) return rc;
  dim3 grid((a.M + GT_M - 1) / GT_M, a.N / BN, L * a.ksplit);
  kern<<<grid, 128, GtTile<BN>::SMEM, st>>>(b);
  XT_CHECK_LAUNCH("k_gemm_tc");
  return XT_OK;
}

template <int TA, int TB, int EPI>
static int gemm(const GemmArgs& a, int L, cudaStream_t st) {
  XT_REQUIRE(a.M > 0 && a.M % 8 == 0 && (a.N == 64 || a.N == 128) && a.ksplit >= 1 && a.K % (GT_BK * a.ksplit) == 0,
             "GEMM shape %d x %d x %d (split %d) not tileable", a.M, a.N, a.K, a.ksplit);
  XT_REQUIRE((a.lda % 8) == 0 && (a.ldb % 8) == 0 && (a.ldc % 4) == 0, "GEMM leading dimensions must allow 16-byte rows");
  return a.N == 64 ? gemm_bn<TA, TB, EPI, 64>(a, L, st) : gemm_bn<TA, TB, EPI, 128>(a, L, st);
}

static int mlp_forward_gemms(MlpHandle* h, const MlpWork& w, int B, cudaStream_t st) {
  const int L = h->L, ps = h->psize;
  int rc;
  GemmArgs a{};
  a.A = w.H1; a.lda = HID; a.sA = (long long)B * HID;
  a.B = h->wb + MlpLayout::W2; a.ldb = HID; a.sB = ps;
  a.M = B; a.N = HID; a.K = HID; a.ksplit = 1;
  a.C = w.Z2; a.ldc = HID; a.sC = (long long)B * HID; a.bias = h->params + MlpLayout::B2; a.sBias = ps;
  a.Hout = w.H2;
  if ((rc = gemm<0, 0, EPI_BIAS_SILU>(a, L, st))) return rc;
  a.A = w.H2; a.B = h->wb + MlpLayout::W3; a.C = w.Z3; a.bias = h->params + MlpLayout::B3; a.Hout = w.H3;
  if ((rc = gemm<0, 0, EPI_BIAS_SILU>(a, L, st))) return rc;
  GemmArgs y{};
  y.A = w.H3; y.lda = HID; y.sA = (long long)B * HID;
  y.B = h->wb + MlpLayout::W4; y.ldb = HID; y.sB = ps;
  y.M = B; y.N = NOP; y.K = HID; y.ksplit = 1;
  y.C = w.Y; y.ldc = NOP; y.sC = (long long)B * NOP; y.bias = h->params + MlpLayout::B4; y.sBias = ps;
  return gemm<0, 0, EPI_BIAS>(y, L, st);
}

static void free_mlp(MlpHandle* h) {
  if (!h) return;
  cudaFree(h->params);
  cudaFree(h->grads);
  cudaFree(h->m1);
  cudaFree(h->m2);
  cudaFree(h->wb);
  delete h;
}

static int check_batch(MlpHandle* h, int B, void* workspace, size_t workspace_bytes, MlpWork* w) {
  XT_REQUIRE(B > 0 && B % 64 == 0, "batch must be a positive multiple of 64 (got %d)", B);
  *w = mlp_work(workspace, h->L, B);
  if (!workspace || workspace_bytes < w->total) {
    set_error("workspace of %zu bytes needed, %zu given", w->total, workspace_bytes);
    return XT_ERR_WORKSPACE;
  }
  return XT_OK;
}

bool mlp_view(void* handle, MlpHandle** out) {
  *out = static_cast<MlpHandle*>(handle);
  return *out != nullptr;
}

}  // namespace xt

using namespace xt;

extern "C" {

int xt_mlp_param_size(void) { return MlpLayout::SIZE; }

int xt_mlp_create(int L, int nout, const float* init_params, void** handle) {
  XT_REQUIRE(handle, "NULL handle out-pointer");
  *handle = nullptr;
  XT_REQUIRE(L >= 1 && L <= MLP_LMAX + 1, "need 1 <= L <= %d networks (got %d)", MLP_LMAX + 1, L);
  XT_REQUIRE(nout >= 2 && nout <= NOP && nout % 2 == 0, "need an even 2 <= nout <= %d (got %d)", NOP, nout);
  XT_REQUIRE(init_params, "initial parameters required (L x xt_mlp_param_size floats)");
  MlpHandle* h = new MlpHandle();
  h->L = L;
  h->nout = nout;
  h->psize = MlpLayout::SIZE;
  const size_t n = (size_t)L * h->psize;
  cudaError_t e = cudaMalloc((void**)&h->params, n * 4);
  if (e == cudaSuccess) e = cudaMalloc((void**)&h->grads, n * 4);
  if (e == cudaSuccess) e = cudaMalloc((void**)&h->m1, n * 4);
  if (e == cudaSuccess) e = cudaMalloc((void**)&h->m2, n * 4);
  if (e == cudaSuccess) e = cudaMalloc((void**)&h->wb, n * 2);
  if (e == cudaSuccess) e = cudaMemcpy(h->params, init_params, n * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(h->m1, 0, n * 4);
  if (e == cudaSuccess) e = cudaMemset(h->m2, 0, n * 4);
  if (e == cudaSuccess) e = cudaMemset(h->grads, 0, n * 4);
  if (e == cudaSuccess) {
    k_mlp_refresh<<<grid_for((long long)n, 256, 4), 256>>>(h->params, h->wb, (int)n, h->psize, nout);
    e = cudaDeviceSynchronize();
  }
  if (e != cudaSuccess) {
    free_mlp(h);
    return cuda_fail(e, "xt_mlp_create");
  }
  *handle = h;
  return XT_OK;
}

int xt_mlp_destroy(void* handle) {
  free_mlp(static_cast<MlpHandle*>(handle));
  return XT_OK;
}

size_t xt_mlp_workspace(void* handle, int B) {
  MlpHandle* h = static_cast<MlpHandle*>(handle);
  if (!h || B <= 0) return 0;
  return mlp_work(nullptr, h->L, B).total;
}

int xt_mlp_get(void* handle, int which, float* host_out) {
  MlpHandle* h = static_cast<MlpHandle*>(handle);
  XT_REQUIRE(h && host_out, "NULL handle or output");
  XT_REQUIRE(which >= 0 && which <= 3, "which: 0 params, 1 grads, 2 Adam m, 3 Adam v");
  const float* src = which == 0 ? h->params : which == 1 ? h->grads : which == 2 ? h->m1 : h->m2;
  XT_CUDA(cudaDeviceSynchronize());
  XT_CUDA(cudaMemcpy(host_out, src, (size_t)h->L * h->psize * 4, cudaMemcpyDeviceToHost));
  return XT_OK;
}

int xt_mlp_set_params(void* handle, const float* host_params, long long step) {
  MlpHandle* h = static_cast<MlpHandle*>(handle);
  XT_REQUIRE(h && host_params, "NULL handle or parameters");
  const size_t n = (size_t)h->L * h->psize;
  XT_CUDA(cudaDeviceSynchronize());
  XT_CUDA(cudaMemcpy(h->params, host_params, n * 4, cudaMemcpyHostToDevice));
  XT_CUDA(cudaMemset(h->m1, 0, n * 4));
  XT_CUDA(cudaMemset(h->m2, 0, n * 4));
  h->step = step;
  k_mlp_refresh<<<grid_for((long long)n, 256, 4), 256>>>(h->params, h->wb, (int)n, h->psize, h->nout);
  XT_CHECK_LAUNCH("k_mlp_refresh");
  XT_CUDA(cudaDeviceSynchronize());
  return XT_OK;
}

int xt_mlp_forward(void* handle, const float* t, int B, float* Y, void* workspace, size_t workspace_bytes,
                   void* stream) {
  MlpHandle* h = static_cast<MlpHandle*>(handle);
  XT_REQUIRE(h && t && Y, "NULL argument");
  MlpWork w;
  int rc = check_batch(h, B, workspace, workspace_bytes, &w);
  if (rc) return rc;
  w.Y = Y;
  cudaStream_t st = as_stream(stream);
  k_mlp_l1_fwd<<<dim3(grid_for((long long)B * HID, 256, 4), h->L), 256, 0, st>>>(h->params, h->psize, t, B, w.Z1,
                                                                                 w.H1);
  XT_CHECK_LAUNCH("k_mlp_l1_fwd");
  return mlp_forward_gemms(h, w, B, st);
}

int xt_mlp_train_step(void* handle, const float* t, const float* T, long long ldT, int B, float lr, int do_update,
                      double* loss_out, void* workspace, size_t workspace_bytes, void* stream) {
  MlpHandle* h = static_cast<MlpHandle*>(handle);
  XT_REQUIRE(h && t && T, "NULL argument");
  XT_REQUIRE(ldT >= (long long)B * NOP, "target stride %lld below batch x %d", ldT, NOP);
  MlpWork w;
  int rc = check_batch(h, B, workspace, workspace_bytes, &w);
  if (rc) return rc;
  cudaStream_t st = as_stream(stream);
  const int L = h->L, ps = h->psize;
  k_mlp_l1_fwd<<<dim3(grid_for((long long)B * HID, 256, 4), L), 256, 0, st>>>(h->params, ps, t, B, w.Z1, w.H1);
  XT_CHECK_LAUNCH("k_mlp_l1_fwd");
  if ((rc = mlp_forward_gemms(h, w, B, st))) return rc;
  XT_CUDA(cudaMemsetAsync(w.loss, 0, L * sizeof(double), st));
  k_mlp_loss<<<dim3(grid_for((long long)B * NOP, 256, 4), L), 256, 0, st>>>(w.Y, T, ldT, B, h->nout, w.dY, w.dYb,
                                                                            w.loss);
  XT_CHECK_LAUNCH("k_mlp_loss");
  XT_CUDA(cudaMemsetAsync(h->grads, 0, (size_t)L * ps * 4, st));
  int ksp = 1;
  while (ksp < 32 && B % (32 * ksp * 2) == 0 && B / (ksp * 2) >= 256) ksp *= 2;
  // dW4[o][k] = sum_b dY[b][o] H3[b][k]
  GemmArgs g{};
  g.A = w.dYb; g.lda = NOP; g.sA = (long long)B * NOP;
  g.B = w.H3; g.ldb = HID; g.sB = (long long)B * HID;
  g.M = NOP; g.N = HID; g.K = B; g.ksplit = ksp;
  g.C = h->grads + MlpLayout::W4; g.ldc = HID; g.sC = ps;
  if ((rc = gemm<1, 1, EPI_ATOMIC>(g, L, st))) return rc;
  k_mlp_bias_grad<<<dim3(NOP, L), 256, 0, st>>>(w.dY, B, NOP, h->nout, h->grads, ps, MlpLayout::B4);
  XT_CHECK_LAUNCH("k_mlp_bias_grad");
  // dH3 = dY W4, dZ3 = dH3 silu'(Z3)
  GemmArgs d{};
  d.A = w.dYb; d.lda = NOP; d.sA = (long long)B * NOP;
  d.B = h->wb + MlpLayout::W4; d.ldb = HID; d.sB = ps;
  d.M = B; d.N = HID; d.K = NOP; d.ksplit = 1;
  d.C = w.dZ3; d.ldc = HID; d.sC = (long long)B * HID; d.Hout = w.dZ3b; d.Zsaved = w.Z3;
  if ((rc = gemm<0, 1, EPI_DSILU>(d, L, st))) return rc;
  // dW3 = dZ3^T H2, db3
  g.A = w.dZ3b; g.lda = HID; g.sA = (long long)B * HID;
  g.B = w.H2; g.M = HID; g.C = h->grads + MlpLayout::W3;
  if ((rc = gemm<1, 1, EPI_ATOMIC>(g, L, st))) return rc;
  k_mlp_bias_grad<<<dim3(HID, L), 256, 0, st>>>(w.dZ3, B, HID, HID, h->grads, ps, MlpLayout::B3);
  XT_CHECK_LAUNCH("k_mlp_bias_grad");
  // dH2 = dZ3 W3, dZ2
  d.A = w.dZ3b; d.lda = HID; d.sA = (long long)B * HID;
  d.B = h->wb + MlpLayout::W3; d.K = HID;
  d.C = w.dZ2; d.Hout = w.dZ2b; d.Zsaved = w.Z2;
  if ((rc = gemm<0, 1, EPI_DSILU>(d, L, st))) return rc;
  // dW2 = dZ2^T H1, db2
  g.A = w.dZ2b; g.B = w.H1; g.C = h->grads + MlpLayout::W2;
  if ((rc = gemm<1, 1, EPI_ATOMIC>(g, L, st))) return rc;
  k_mlp_bias_grad<<<dim3(HID, L), 256, 0, st>>>(w.dZ2, B, HID, HID, h->grads, ps, MlpLayout::B2);
  XT_CHECK_LAUNCH("k_mlp_bias_grad");
  // dH1 = dZ2 W2, dZ1 (its BF16 copy is not used; dZ3b is free scratch by now)
  d.A = w.dZ2b; d.B = h->wb + MlpLayout::W2; d.C = w.dZ1; d.Hout = w.dZ3b; d.Zsaved = w.Z1;
  if ((rc = gemm<0, 1, EPI_DSILU>(d, L, st))) return rc;
  k_mlp_l1_bwd<<<dim3(HID, L), 256, 0, st>>>(w.dZ1, t, B, h->grads, ps);
  XT_CHECK_LAUNCH("k_mlp_l1_bwd");
  if (loss_out) XT_CUDA(cudaMemcpyAsync(loss_out, w.loss, L * sizeof(double), cudaMemcpyDeviceToDevice, st));
  if (do_update) {
    h->step += 1;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f - powf(b1, (float)h->step), c2 = 1.f - powf(b2, (float)h->step);
    const int total = L * ps;
    k_mlp_adam<<<grid_for(total, 256, 4), 256, 0, st>>>(h->params, h->grads, h->m1, h->m2, h->wb, total, ps, h->nout,
                                                       lr, b1, b2, eps, c1, c2);
    XT_CHECK_LAUNCH("k_mlp_adam");
  }
  return XT_OK;
}

int xt_mlp_labels(void* sph, int K, const double* r, long long n, double a_prior, const double* s, const double* sig,
                  double c0, double c1, float* t_out, float* T_out, long long ldT, void* stream) {
  SphTab<double> T;
  SphTab<float> Tf;
  XT_REQUIRE(sph_tabs(sph, &T, &Tf), "NULL SL table handle");
  const double* efp = nullptr;
  sph_efp(sph, &efp);
  XT_REQUIRE(T.cmap == 2, "the learned radial basis needs a logarithmic (cmap 2) SL table");
  XT_REQUIRE(T.lmax <= MLP_LMAX, "learned radial basis: lmax <= %d", MLP_LMAX);
  XT_REQUIRE(K >= 1 && K <= T.nmax && 2 * K <= NOP, "need 1 <= K <= min(nmax, %d)", NOP / 2);
  XT_REQUIRE(r && s && sig && t_out && T_out && n >= 0, "NULL argument");
  XT_REQUIRE(ldT >= n * NOP, "target stride below n x %d", NOP);
  XT_REQUIRE(a_prior > 0.0, "prior scale must be positive");
  if (n == 0) return XT_OK;
  const double rmin = exp((double)T.lo), rmax = exp((double)T.hi);
  k_mlp_labels<<<grid_for(n, 128, 8), 128, 0, as_stream(stream)>>>(T, efp, K, r, n, a_prior, s, sig, rmin, rmax, c0,
                                                                  c1, t_out, T_out, ldT);
  XT_CHECK_LAUNCH("k_mlp_labels");
  return XT_OK;
}

}  // extern "C"
