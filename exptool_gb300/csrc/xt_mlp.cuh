// Learned radial basis: shared definitions of the per-l networks (training in
// xt_mlp.cu, inference in xt_mlp_eval.cu).
//
// Network for harmonic l (all l networks are batched):
//   t = clamp((ln r - c0) * c1, -1, 1)
//   H1 = silu(t W1 + b1), H2 = silu(H1 W2^T + b2), H3 = silu(H2 W3^T + b3)
//   Y  = H3 W4^T + b4      (Y[n] and Y[K+n], n < K: residuals of phi_nl and r dphi_nl/dr)
// The radial functions are phi_nl(r) = s_nl HO_nl(r) + sigma_nl Y[n] and
// r dphi_nl/dr = s_nl r dHO_nl/dr + sigma'_nl Y[K+n], with HO_nl the
// Hernquist-Ostriker functions (an analytic prior for a Hernquist-like
// background) and s, sigma per-function scales fitted on the host.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "xt_internal.cuh"

namespace xt {

constexpr int MLP_HID = 128;   // hidden width
constexpr int MLP_NOP = 64;    // output width padded (2K <= 64)
constexpr int MLP_NC = 32;     // contracted outputs per l: 2 (2l+1) <= 32, l <= 7
constexpr int MLP_WPAD = MLP_HID + 8;   // shared-memory row pitch (bf16): conflict-free ldmatrix
constexpr int MLP_LMAX = 7;
constexpr int MLP_KMAX = 32;

// Parameter offsets (elements) inside one network's block; FP32 masters and
// BF16 copies share the layout.
struct MlpLayout {
  static constexpr int W1 = 0;                             // [HID]
  static constexpr int B1 = W1 + MLP_HID;                  // [HID]
  static constexpr int W2 = B1 + MLP_HID;                  // [HID][HID]  (out, in)
  static constexpr int B2 = W2 + MLP_HID * MLP_HID;        // [HID]
  static constexpr int W3 = B2 + MLP_HID;                  // [HID][HID]
  static constexpr int B3 = W3 + MLP_HID * MLP_HID;        // [HID]
  static constexpr int W4 = B3 + MLP_HID;                  // [NOP][HID]
  static constexpr int B4 = W4 + MLP_NOP * MLP_HID;        // [NOP]
  static constexpr int SIZE = B4 + MLP_NOP;
};
static_assert((MlpLayout::SIZE * 2) % 16 == 0, "network block must keep 16-byte alignment of bf16 copies");
static_assert((MlpLayout::W2 * 2) % 16 == 0 && (MlpLayout::W3 * 2) % 16 == 0 && (MlpLayout::W4 * 2) % 16 == 0,
              "weight matrices must start on 16-byte boundaries");

struct MlpHandle {
  int L, nout;
  int psize;
  float* params = nullptr;        // [L][psize] FP32 masters
  float* grads = nullptr;
  float* m1 = nullptr;
  float* m2 = nullptr;
  __nv_bfloat16* wb = nullptr;    // [L][psize] BF16 copies used by the products
  long long step = 0;
};

constexpr int TC_MAX_BANDS = 64;

// Arguments of the tensor-memory network pass (xt_mlp_tc.cu).
struct TcArgs {
  const float4* xyzw;
  long long n;
  const __nv_bfloat16* wb;
  const float* params;
  int psize, L;
  const __nv_bfloat16* w4h;
  const __nv_bfloat16* w4l;
  const float* b4c;
  float c0, c1, rmin, rmax;
  float lnr0, inv_bw;
  int nb;
  float* R;
  int rstride;
  int* err;                   // set to 1 on an MMA wait timeout
  const float* CS;            // [(lmax+1)^2][K] prior weights c * scale * s (adds the prior to R)
  int K;
  float a_inv;                // 1 / prior scale length
  int band_use[TC_MAX_BANDS];
};
int launch_mlp_radial_tc(const TcArgs& a, int nsm, cudaStream_t st);
int tc_error_flag(int** dptr);

// SiLU through the hardware tanh: sigma(z) = (1 + tanh(z/2)) / 2.  Training,
// the gradients and both inference engines use these same functions, so the
// trained network is the evaluated one.  (Packed-half tanh halves the
// transcendental instructions but costs more conversions than it saves here.)
__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sigm_fast(float z) { return fmaf(0.5f, tanh_fast(0.5f * z), 0.5f); }
// silu(z) = h + h tanh(h) with h = z/2.  Halving is exact, so callers may
// form h directly as fma(x, w/2, b/2) = (x w + b)/2 with the same bits.
__device__ __forceinline__ float silu_h(float h) { return fmaf(h, tanh_fast(h), h); }
__device__ __forceinline__ float silu_fast(float z) { return silu_h(0.5f * z); }
__device__ __forceinline__ float dsilu_fast(float z) {
  const float s = sigm_fast(z);
  return s * fmaf(z, 1.f - s, 1.f);
}
__device__ __forceinline__ float2 silu_fast2(float z0, float z1) { return make_float2(silu_fast(z0), silu_fast(z1)); }

__device__ __forceinline__ unsigned pack_bf16x2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<unsigned*>(&v);
}
__device__ __forceinline__ unsigned pack_bf16x2(float2 v) { return pack_bf16x2(v.x, v.y); }

// D += A(16x16, row) * B(16x8, col), BF16 in, FP32 accumulate.
__device__ __forceinline__ void mma_bf16_16816(float d[4], const unsigned a[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldsm_x4(unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3, const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}

// Hernquist-Ostriker radial functions (Hernquist & Ostriker 1992, eq. 2.12
// up to normalisation) in units u = r/a:
//   HO_nl(u)       = -u^l / (1+u)^(2l+1) C_n^(2l+3/2)(xi),  xi = (u-1)/(u+1)
//   u dHO_nl/du    = -u^l / (1+u)^(2l+1) [ (l - (2l+1) u/(1+u)) C_n + 2u/(1+u)^2 dC_n/dxi ]
// Gegenbauer polynomials by the three-term recurrence
//   n C_n^a = 2 (n+a-1) xi C_{n-1}^a - (n+2a-2) C_{n-2}^a,
// and dC_n^a/dxi = 2a C_{n-1}^(a+1) by the same recurrence at a+1.
// Calls f(n, HO_nl, u dHO_nl/du) for n = 0..K-1.
template <typename R, typename F>
__device__ __forceinline__ void ho_radial(R u, int l, int K, const R* inv_n, F&& f) {
  const R inv1u = R(1) / (R(1) + u);
  const R xi = (u - R(1)) * inv1u;
  R pre = inv1u;
  for (int i = 0; i < l; ++i) pre *= u * inv1u * inv1u;   // u^l / (1+u)^(2l+1)
  const R g1 = R(l) - R(2 * l + 1) * u * inv1u;
  const R g2 = R(2) * u * inv1u * inv1u;
  const R a = R(2 * l) + R(1.5);
  R c1 = R(0), c2 = R(0);     // C_{n-1}, C_{n-2}
  R d1 = R(0), d2 = R(0);     // C^(a+1)_{n-2}, C^(a+1)_{n-3}  (derivative uses C^(a+1)_{n-1})
  for (int n = 0; n < K; ++n) {
    R c, dc;
    if (n == 0) {
      c = R(1);
      dc = R(0);
    } else if (n == 1) {
      c = R(2) * a * xi;
      dc = R(2) * a;          // 2a C_0^(a+1)
      d1 = R(1);
    } else {
      c = (R(2) * (R(n) + a - R(1)) * xi * c1 - (R(n) + R(2) * a - R(2)) * c2) * inv_n[n];
      // C^(a+1)_{n-1} from its recurrence (index k = n-1 >= 1)
      const int k = n - 1;
      R dk;
      if (k == 1) dk = R(2) * (a + R(1)) * xi;
      else dk = (R(2) * (R(k) + a) * xi * d1 - (R(k) + R(2) * a) * d2) * inv_n[k];
      d2 = d1;
      d1 = dk;
      dc = R(2) * a * dk;
    }
    c2 = c1;
    c1 = c;
    f(n, -pre * c, -pre * (g1 * c + g2 * dc));
  }
}

}  // namespace xt
