// Learned radial basis, part 2: force evaluation with the trained networks.
//
// Pass 1 (k_mlp_radial, tensor cores): for every point and every l, the
// network's residual radial functions contracted with the coefficients.  The
// contraction is folded into the last layer on the host side of the pass
// (W4c[row] = sum_n c[row,n] sigma_n W4[n], split into BF16 hi + lo so the
// folded weights keep ~16 bits), so one MMA chain per l yields, per
// coefficient row, sum_n c sigma Y_n (potential) and its r d/dr partner.  Each
// warp carries 16 points through all layers in registers: the FP32
// accumulator fragment of one layer becomes, after bias + SiLU + BF16
// packing, the A fragment of the next (m16n8k16 C and A layouts coincide per
// 16-column slice), and only the weights live in shared memory (ldmatrix).
//
// Pass 2 (k_learned_eval, FP32 CUDA cores): per point, the analytic
// Hernquist-Ostriker prior contracted with c*s (unless pass 1 added it),
// plus the pass-1 sums, assembled with the associated Legendre functions and
// cos/sin(m phi) as in spheresl.all_eval (spheresl.py:987-1102).  Points in radius bands marked
// for the table fall back to FP32 table interpolation of the coefficient-
// contracted field (the mixed-precision table path).
#include <cmath>

#include "xt_launch.cuh"
#include "xt_mlp.cuh"

namespace xt {

constexpr int HID = MLP_HID;
constexpr int NC = MLP_NC;
constexpr int WPAD = MLP_WPAD;
constexpr int RAD_WARPS = 8;
constexpr int MAX_BANDS = 64;

bool mlp_view(void* handle, MlpHandle** out);

static size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

struct PrepLayout {
  size_t w4h, w4l, b4c, cs, total;
};

static PrepLayout prep_layout(int L, int K) {
  PrepLayout p{};
  size_t o = 0;
  p.w4h = o; o += al((size_t)L * NC * HID * 2);
  p.w4l = o; o += al((size_t)L * NC * HID * 2);
  p.b4c = o; o += al((size_t)L * NC * 4);
  p.cs = o;  o += al((size_t)L * L * K * 4);
  p.total = o;
  return p;
}

static int r_stride(int lmax) { return (2 * (lmax + 1) * (lmax + 1) + 3) & ~3; }

// Folded last layer and prior coefficients for one coefficient set.
__global__ void __launch_bounds__(256) k_learned_prep(const float* __restrict__ params,
                                                      const __nv_bfloat16* __restrict__ wb, int psize, int K,
                                                      const double* __restrict__ coef, int nmax, double scale,
                                                      const double* __restrict__ s, const double* __restrict__ sig,
                                                      __nv_bfloat16* __restrict__ w4h, __nv_bfloat16* __restrict__ w4l,
                                                      float* __restrict__ b4c, float* __restrict__ CS) {
  const int l = blockIdx.x;
  const int nout = 2 * (2 * l + 1);
  const float* pl = params + (size_t)l * psize;
  const __nv_bfloat16* wl = wb + (size_t)l * psize;
  for (int i = threadIdx.x; i < NC * HID; i += blockDim.x) {
    const int o = i / HID, k = i % HID;
    double acc = 0.0;
    if (o < nout) {
      const int rr = o >> 1, kind = o & 1, row = l * l + rr;
      for (int n = 0; n < K; ++n)
        acc += coef[(size_t)row * nmax + n] * scale * sig[l * 2 * K + kind * K + n] *
               (double)__bfloat162float(wl[MlpLayout::W4 + (kind * K + n) * HID + k]);
    }
    const __nv_bfloat16 hi = __float2bfloat16_rn((float)acc);
    const __nv_bfloat16 lo = __float2bfloat16_rn((float)(acc - (double)__bfloat162float(hi)));
    w4h[((size_t)l * NC + o) * HID + k] = hi;
    w4l[((size_t)l * NC + o) * HID + k] = lo;
  }
  for (int o = threadIdx.x; o < NC; o += blockDim.x) {
    double acc = 0.0;
    if (o < nout) {
      const int rr = o >> 1, kind = o & 1, row = l * l + rr;
      for (int n = 0; n < K; ++n)
        acc += coef[(size_t)row * nmax + n] * scale * sig[l * 2 * K + kind * K + n] *
               (double)pl[MlpLayout::B4 + kind * K + n];
    }
    b4c[l * NC + o] = (float)acc;
  }
  for (int i = threadIdx.x; i < (2 * l + 1) * K; i += blockDim.x) {
    const int rr = i / K, n = i % K, row = l * l + rr;
    CS[(size_t)row * K + n] = (float)(coef[(size_t)row * nmax + n] * scale * s[l * K + n]);
  }
}

struct RadialArgs {
  const float4* xyzw;
  long long n;
  const __nv_bfloat16* wb;
  const float* params;
  int psize;
  const __nv_bfloat16* w4h;
  const __nv_bfloat16* w4l;
  const float* b4c;
  float c0, c1, rmin, rmax;
  float lnr0, inv_bw;
  int nb;
  float* R;
  int rstride;
  int band_use[MAX_BANDS];
};

// One hidden layer for the warp's 16 rows: A (16 x 128, BF16 fragments) ->
// silu(A W^T + b) in the same fragment layout.
__device__ __forceinline__ void hidden_layer(unsigned (&A)[8][4], const __nv_bfloat16* Ws, const float* bias,
                                             int lane) {
  const int tq = lane & 3, q = lane >> 3, r8 = lane & 7;
  float acc[16][4];
#pragma unroll
  for (int j = 0; j < 16; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[j][e] = 0.f;
  const __nv_bfloat16* base = Ws + ((q >> 1) * 8 + r8) * WPAD + (q & 1) * 8;
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) {
#pragma unroll
    for (int jp = 0; jp < 8; ++jp) {
      unsigned b0, b1, b2, b3;
      ldsm_x4(b0, b1, b2, b3, base + 16 * jp * WPAD + 16 * kk);
      mma_bf16_16816(acc[2 * jp], A[kk], b0, b1);
      mma_bf16_16816(acc[2 * jp + 1], A[kk], b2, b3);
    }
  }
#pragma unroll
  for (int kk = 0; kk < 8; ++kk) {
    const int c0 = 16 * kk + 2 * tq, c1 = c0 + 8;
    const float p0 = bias[c0], p1 = bias[c0 + 1], p2 = bias[c1], p3 = bias[c1 + 1];
    A[kk][0] = pack_bf16x2(silu_fast2(acc[2 * kk][0] + p0, acc[2 * kk][1] + p1));
    A[kk][1] = pack_bf16x2(silu_fast2(acc[2 * kk][2] + p0, acc[2 * kk][3] + p1));
    A[kk][2] = pack_bf16x2(silu_fast2(acc[2 * kk + 1][0] + p2, acc[2 * kk + 1][1] + p3));
    A[kk][3] = pack_bf16x2(silu_fast2(acc[2 * kk + 1][2] + p2, acc[2 * kk + 1][3] + p3));
  }
}

// Radius of a point with an explicit FMA order: both passes must agree on
// every point's band.
__device__ __forceinline__ float point_radius(float4 v) { return sqrtf(fmaf(v.x, v.x, fmaf(v.y, v.y, v.z * v.z))); }

__device__ __forceinline__ int band_of(float lr, float lnr0, float inv_bw, int nb) {
  int b = (int)((lr - lnr0) * inv_bw);
  return b < 0 ? 0 : (b >= nb ? nb - 1 : b);
}

// grid (gx, L): blockIdx.y = l; the CTA stages network l once and walks
// 16-point warp tiles.  Writes R[p][2 (l^2 + rr) + {0,1}] for rr <= 2l.
__global__ void __launch_bounds__(RAD_WARPS * 32, 2) k_mlp_radial(RadialArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __nv_bfloat16* W2s = reinterpret_cast<__nv_bfloat16*>(smem);
  __nv_bfloat16* W3s = W2s + HID * WPAD;
  __nv_bfloat16* W4h = W3s + HID * WPAD;
  __nv_bfloat16* W4l = W4h + NC * WPAD;
  float* w1 = reinterpret_cast<float*>(W4l + NC * WPAD);
  float* b1 = w1 + HID;
  float* b2 = b1 + HID;
  float* b3 = b2 + HID;
  float* b4 = b3 + HID;
  const int l = blockIdx.y;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const __nv_bfloat16* gw = a.wb + (size_t)l * a.psize;
  const float* gp = a.params + (size_t)l * a.psize;
  for (int i = tid; i < HID * HID / 8; i += blockDim.x) {
    const int row = i >> 4, c8 = (i & 15) * 8;
    *reinterpret_cast<uint4*>(W2s + row * WPAD + c8) =
        *reinterpret_cast<const uint4*>(gw + MlpLayout::W2 + row * HID + c8);
    *reinterpret_cast<uint4*>(W3s + row * WPAD + c8) =
        *reinterpret_cast<const uint4*>(gw + MlpLayout::W3 + row * HID + c8);
  }
  for (int i = tid; i < NC * HID / 8; i += blockDim.x) {
    const int row = i >> 4, c8 = (i & 15) * 8;
    const size_t g = ((size_t)l * NC + row) * HID + c8;
    *reinterpret_cast<uint4*>(W4h + row * WPAD + c8) = *reinterpret_cast<const uint4*>(a.w4h + g);
    *reinterpret_cast<uint4*>(W4l + row * WPAD + c8) = *reinterpret_cast<const uint4*>(a.w4l + g);
  }
  for (int i = tid; i < HID; i += blockDim.x) {
    w1[i] = gp[MlpLayout::W1 + i];
    b1[i] = gp[MlpLayout::B1 + i];
    b2[i] = gp[MlpLayout::B2 + i];
    b3[i] = gp[MlpLayout::B3 + i];
  }
  for (int i = tid; i < NC; i += blockDim.x) b4[i] = a.b4c[l * NC + i];
  __syncthreads();
  const int* use = a.band_use;

  const int gq = lane >> 2, tq = lane & 3, q = lane >> 3, r8 = lane & 7;
  const int nout = 2 * (2 * l + 1);
  const int col0 = 2 * l * l;
  const long long ntile = (a.n + 15) >> 4;
  for (long long tile = (long long)blockIdx.x * RAD_WARPS + warp; tile < ntile;
       tile += (long long)gridDim.x * RAD_WARPS) {
    const long long p0 = tile * 16 + gq, p1 = p0 + 8;
    const bool v0 = p0 < a.n, v1 = p1 < a.n;
    float r0 = 1.f, r1 = 1.f;
    if (v0) r0 = point_radius(a.xyzw[p0]);
    if (v1) r1 = point_radius(a.xyzw[p1]);
    r0 = fminf(fmaxf(r0, a.rmin), a.rmax);
    r1 = fminf(fmaxf(r1, a.rmin), a.rmax);
    const float lr0 = logf(r0), lr1 = logf(r1);
    const bool u0 = v0 && use[band_of(lr0, a.lnr0, a.inv_bw, a.nb)];
    const bool u1 = v1 && use[band_of(lr1, a.lnr0, a.inv_bw, a.nb)];
    if (!__any_sync(0xffffffffu, u0 || u1)) continue;
    const float t0 = fminf(fmaxf((lr0 - a.c0) * a.c1, -1.f), 1.f);
    const float t1 = fminf(fmaxf((lr1 - a.c0) * a.c1, -1.f), 1.f);
    unsigned A[8][4];
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
      const int c = 16 * kk + 2 * tq, d = c + 8;
      A[kk][0] = pack_bf16x2(silu_fast2(fmaf(t0, w1[c], b1[c]), fmaf(t0, w1[c + 1], b1[c + 1])));
      A[kk][1] = pack_bf16x2(silu_fast2(fmaf(t1, w1[c], b1[c]), fmaf(t1, w1[c + 1], b1[c + 1])));
      A[kk][2] = pack_bf16x2(silu_fast2(fmaf(t0, w1[d], b1[d]), fmaf(t0, w1[d + 1], b1[d + 1])));
      A[kk][3] = pack_bf16x2(silu_fast2(fmaf(t1, w1[d], b1[d]), fmaf(t1, w1[d + 1], b1[d + 1])));
    }
    hidden_layer(A, W2s, b2, lane);
    hidden_layer(A, W3s, b3, lane);
    float o[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) o[j][e] = 0.f;
    const int boff = ((q >> 1) * 8 + r8) * WPAD + (q & 1) * 8;
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
#pragma unroll
      for (int jp = 0; jp < 2; ++jp) {
        unsigned h0, h1, h2, h3, e0, e1, e2, e3;
        ldsm_x4(h0, h1, h2, h3, W4h + boff + 16 * jp * WPAD + 16 * kk);
        ldsm_x4(e0, e1, e2, e3, W4l + boff + 16 * jp * WPAD + 16 * kk);
        mma_bf16_16816(o[2 * jp], A[kk], h0, h1);
        mma_bf16_16816(o[2 * jp + 1], A[kk], h2, h3);
        mma_bf16_16816(o[2 * jp], A[kk], e0, e1);
        mma_bf16_16816(o[2 * jp + 1], A[kk], e2, e3);
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = 8 * j + 2 * tq;
      if (col < nout) {
        const float bb0 = b4[col], bb1 = b4[col + 1];
        if (u0) *reinterpret_cast<float2*>(a.R + p0 * a.rstride + col0 + col) = make_float2(o[j][0] + bb0, o[j][1] + bb1);
        if (u1) *reinterpret_cast<float2*>(a.R + p1 * a.rstride + col0 + col) = make_float2(o[j][2] + bb0, o[j][3] + bb1);
      }
    }
  }
}

struct LearnArgs {
  SphTab<float> T;
  const float* GH;          // FP32 coefficient-contracted table field (SphFieldLayout<float>)
  const float* CS;          // [nrow][K] c * scale * s
  const float* R;           // pass-1 sums [n][rstride]
  int rstride, K, lmax, no_odd;
  float a_inv, rmin, rmax, lnr0, inv_bw;
  int nb;
  const float4* xyzw;
  long long n;
  float4* out;              // pot, dpot/dr, dpot/dcos(theta), dpot/dphi
  int prior_in_R;           // pass 1 already added the prior (tensor-memory engine)
  int band_use[MAX_BANDS];
};

template <int LCAP>
__global__ void __launch_bounds__(256) k_learned_eval(LearnArgs a) {
  extern __shared__ float shm[];
  const int nrow = (a.lmax + 1) * (a.lmax + 1);
  float* CS = shm;
  float* inv_n = CS + nrow * a.K;
  for (int i = threadIdx.x; i < nrow * a.K; i += blockDim.x) CS[i] = a.CS[i];
  for (int i = threadIdx.x; i < MLP_KMAX; i += blockDim.x) inv_n[i] = i ? 1.f / (float)i : 0.f;
  __syncthreads();
  const int* use = a.band_use;
  const int lstride = a.T.lmax + 1;
  constexpr int NT = (LCAP + 1) * (LCAP + 2) / 2;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < a.n;
       p += (long long)gridDim.x * blockDim.x) {
    const float4 v = a.xyzw[p];
    const float r = point_radius(v);
    const float costh = r > 0.f ? v.z / r : 0.f;
    float c1, s1;
    unit_phi(v.x, v.y, c1, s1);
    const float rc = fminf(fmaxf(r, a.rmin), a.rmax);
    const bool net = use[band_of(logf(rc), a.lnr0, a.inv_bw, a.nb)] != 0;
    float P[NT], dP[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) { P[k] = 0.f; dP[k] = 0.f; }
    legendre<float, LCAP>(costh, a.lmax, P);
    dlegendre<float, LCAP>(costh, a.lmax, P, dP);
    float cm[LCAP + 1], sm[LCAP + 1];
    multiples<float, LCAP>(c1, s1, a.lmax, cm, sm);
    SphBins<float> B{};
    if (!net) B = sph_bins(a.T, r, true, false);
    const float* Rp = a.R + p * a.rstride;
    const float inv_rc = 1.f / rc;
    const float u = rc * a.a_inv;
    float pot0 = 0.f, pot1 = 0.f, potr = 0.f, pott = 0.f, potp = 0.f;
#pragma unroll
    for (int l = 0; l <= LCAP; ++l) {
      if (l > a.lmax) break;
      if (a.no_odd && (l & 1)) continue;
      constexpr int RW = 2 * LCAP + 1;
      float pv[RW], dv[RW];
      const int loff = l * l;
      if (net) {
#pragma unroll
        for (int rr = 0; rr < 2 * l + 1; ++rr) {
          const float2 w = *reinterpret_cast<const float2*>(Rp + 2 * (loff + rr));
          pv[rr] = w.x;
          dv[rr] = w.y;
        }
        if (!a.prior_in_R) {
          const float* cs = CS + loff * a.K;
          ho_radial<float>(u, l, a.K, inv_n, [&](int n, float ho, float uho) {
#pragma unroll
            for (int rr = 0; rr < 2 * l + 1; ++rr) {
              const float c = cs[rr * a.K + n];
              pv[rr] = fmaf(c, ho, pv[rr]);
              dv[rr] = fmaf(c, uho, dv[rr]);
            }
          });
        }
#pragma unroll
        for (int rr = 0; rr < 2 * l + 1; ++rr) dv[rr] *= inv_rc;
      } else {
        const float4* ga = reinterpret_cast<const float4*>(a.GH) + (size_t)B.i * nrow;
#pragma unroll
        for (int rr = 0; rr < 2 * l + 1; ++rr) {
          const float4 q = ga[loff + rr];
          pv[rr] = B.lw0 * q.x + B.lw1 * q.y;
          dv[rr] = B.fac * fmaf(B.x2, q.w, q.z);
        }
      }
      if (l == 0) {
        const float f00 = a.T.fact[0];
        pot0 = f00 * pv[0];
        potr = f00 * dv[0];
        continue;
      }
      {
        const float f = a.T.fact[l * lstride];
        const float fP = f * P[tri(l, 0)];
        pot1 += fP * pv[0];
        potr += fP * dv[0];
        pott += f * dP[tri(l, 0)] * pv[0];
      }
#pragma unroll
      for (int m = 1; m <= l; ++m) {
        const float f = a.T.fact[l * lstride + m];
        const float c = cm[m], s = sm[m];
        const float fP = f * P[tri(l, m)];
        const float angp = pv[2 * m - 1] * c + pv[2 * m] * s;
        pot1 += fP * angp;
        potr += fP * (dv[2 * m - 1] * c + dv[2 * m] * s);
        pott += f * dP[tri(l, m)] * angp;
        potp += fP * (float)m * (-pv[2 * m - 1] * s + pv[2 * m] * c);
      }
    }
    a.out[p] = make_float4(pot0 + pot1, potr, pott, potp);
  }
}

template <int LCAP>
static int launch_learned_eval(const LearnArgs& a, size_t shbytes, cudaStream_t st) {
  k_learned_eval<LCAP><<<grid_for(a.n, 256, 8), 256, shbytes, st>>>(a);
  XT_CHECK_LAUNCH("k_learned_eval");
  return XT_OK;
}

// Pass 1 for n points into R (rstride floats per point): engine 0 = mma.sync
// warp tiles (k_mlp_radial), 1 = tcgen05 / tensor memory (k_mlp_radial_tc).
static int radial_pass(const SphTab<double>& T, MlpHandle* h, const void* prep, int K, double a_prior, double c0,
                       double c1, const int* band_use, int nbands, const float* xyzw, long long n, int engine,
                       float* R, cudaStream_t st) {
  const PrepLayout pl = prep_layout(h->L, K);
  const char* pb = static_cast<const char*>(prep);
  const float lnr0 = (float)T.lo, inv_bw = (float)(nbands / (T.hi - T.lo));
  const float rmin = (float)exp((double)T.lo), rmax = (float)exp((double)T.hi);
  bool any_net = false;
  for (int b = 0; b < nbands; ++b) any_net = any_net || band_use[b] != 0;
  if (!any_net || n == 0) return XT_OK;
  int nsm = 152, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (engine == 1) {
    TcArgs ta{};
    ta.xyzw = reinterpret_cast<const float4*>(xyzw);
    ta.n = n;
    ta.wb = h->wb;
    ta.params = h->params;
    ta.psize = h->psize;
    ta.L = h->L;
    ta.w4h = reinterpret_cast<const __nv_bfloat16*>(pb + pl.w4h);
    ta.w4l = reinterpret_cast<const __nv_bfloat16*>(pb + pl.w4l);
    ta.b4c = reinterpret_cast<const float*>(pb + pl.b4c);
    ta.c0 = (float)c0;
    ta.c1 = (float)c1;
    ta.rmin = rmin;
    ta.rmax = rmax;
    ta.lnr0 = lnr0;
    ta.inv_bw = inv_bw;
    ta.nb = nbands;
    ta.R = R;
    ta.rstride = r_stride(T.lmax);
    for (int b = 0; b < nbands; ++b) ta.band_use[b] = band_use[b] != 0;
    ta.CS = nullptr;          // prior in the second pass (faster than in this pass's epilogue)
    ta.K = K;
    ta.a_inv = (float)(1.0 / a_prior);
    int rc = tc_error_flag(&ta.err);
    if (rc) return rc;
    return launch_mlp_radial_tc(ta, nsm, st);
  }
  RadialArgs ra{};
  ra.xyzw = reinterpret_cast<const float4*>(xyzw);
  ra.n = n;
  ra.wb = h->wb;
  ra.params = h->params;
  ra.psize = h->psize;
  ra.w4h = reinterpret_cast<const __nv_bfloat16*>(pb + pl.w4h);
  ra.w4l = reinterpret_cast<const __nv_bfloat16*>(pb + pl.w4l);
  ra.b4c = reinterpret_cast<const float*>(pb + pl.b4c);
  ra.c0 = (float)c0;
  ra.c1 = (float)c1;
  ra.rmin = rmin;
  ra.rmax = rmax;
  for (int b = 0; b < nbands; ++b) ra.band_use[b] = band_use[b] != 0;
  ra.lnr0 = lnr0;
  ra.inv_bw = inv_bw;
  ra.nb = nbands;
  ra.R = R;
  ra.rstride = r_stride(T.lmax);
  const size_t rad_smem = (size_t)(2 * HID + 2 * NC) * WPAD * 2 + (4 * HID + NC) * 4;
  static bool attr_set = false;
  if (!attr_set) {
    XT_CUDA(cudaFuncSetAttribute(k_mlp_radial, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rad_smem));
    attr_set = true;
  }
  const long long ntile = (n + 15) / 16;
  long long gx = (2LL * nsm + h->L - 1) / h->L;
  const long long gmax = (ntile + RAD_WARPS - 1) / RAD_WARPS;
  if (gx > gmax) gx = gmax;
  if (gx < 1) gx = 1;
  k_mlp_radial<<<dim3((unsigned)gx, h->L), RAD_WARPS * 32, rad_smem, st>>>(ra);
  XT_CHECK_LAUNCH("k_mlp_radial");
  return XT_OK;
}

}  // namespace xt

using namespace xt;

extern "C" {

size_t xt_learned_prep_bytes(void* mlp, int K) {
  MlpHandle* h = nullptr;
  if (!mlp_view(mlp, &h) || K < 1) return 0;
  return prep_layout(h->L, K).total;
}

int xt_learned_prepare(void* sph, void* mlp, int K, const double* expcoef, double coef_scale, const double* s,
                       const double* sig, void* prep, size_t prep_bytes, void* stream) {
  SphTab<double> T;
  XT_REQUIRE(sph_tabs(sph, &T, nullptr), "NULL SL table handle");
  MlpHandle* h = nullptr;
  XT_REQUIRE(mlp_view(mlp, &h), "NULL network handle");
  XT_REQUIRE(h->L == T.lmax + 1, "network count %d != lmax + 1 = %d", h->L, T.lmax + 1);
  XT_REQUIRE(T.lmax <= MLP_LMAX, "learned radial basis: lmax <= %d", MLP_LMAX);
  XT_REQUIRE(K >= 1 && K <= T.nmax && h->nout == 2 * K, "K must match the networks (nout = 2K) and nmax");
  XT_REQUIRE(expcoef && s && sig && prep, "NULL argument");
  const PrepLayout pl = prep_layout(h->L, K);
  if (prep_bytes < pl.total) {
    set_error("prepared buffer of %zu bytes needed, %zu given", pl.total, prep_bytes);
    return XT_ERR_WORKSPACE;
  }
  char* b = static_cast<char*>(prep);
  k_learned_prep<<<h->L, 256, 0, as_stream(stream)>>>(
      h->params, h->wb, h->psize, K, expcoef, T.nmax, coef_scale, s, sig,
      reinterpret_cast<__nv_bfloat16*>(b + pl.w4h), reinterpret_cast<__nv_bfloat16*>(b + pl.w4l),
      reinterpret_cast<float*>(b + pl.b4c), reinterpret_cast<float*>(b + pl.cs));
  XT_CHECK_LAUNCH("k_learned_prep");
  return XT_OK;
}

size_t xt_learned_eval_workspace(void* sph, long long n) {
  SphTab<double> T;
  if (!sph_tabs(sph, &T, nullptr) || n < 0) return 0;
  return al((size_t)n * r_stride(T.lmax) * 4);
}

int xt_learned_eval(void* sph, const void* field_f32, void* mlp, const void* prep, int K, double a_prior, double c0,
                    double c1, const int* band_use, int nbands, const float* xyzw, long long n, int no_odd,
                    int engine, float* out, void* workspace, size_t workspace_bytes, void* stream) {
  SphTab<double> T;
  SphTab<float> Tf;
  XT_REQUIRE(sph_tabs(sph, &T, &Tf), "NULL SL table handle");
  MlpHandle* h = nullptr;
  XT_REQUIRE(mlp_view(mlp, &h), "NULL network handle");
  XT_REQUIRE(T.cmap == 2, "the learned radial basis needs a logarithmic (cmap 2) SL table");
  XT_REQUIRE(h->L == T.lmax + 1 && h->nout == 2 * K && K <= T.nmax, "network / table / K mismatch");
  XT_REQUIRE(field_f32 && prep && band_use && xyzw && out, "NULL argument");
  XT_REQUIRE(nbands >= 1 && nbands <= MAX_BANDS, "need 1 <= nbands <= %d", MAX_BANDS);
  XT_REQUIRE(a_prior > 0.0, "prior scale must be positive");
  XT_REQUIRE((reinterpret_cast<uintptr_t>(xyzw) & 15) == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0,
             "xyzw and out must be 16-byte aligned float4 arrays");
  XT_REQUIRE(n >= 0, "negative point count");
  if (n == 0) return XT_OK;
  const size_t need = xt_learned_eval_workspace(sph, n);
  if (!workspace || workspace_bytes < need) {
    set_error("workspace of %zu bytes needed, %zu given", need, workspace_bytes);
    return XT_ERR_WORKSPACE;
  }
  cudaStream_t st = as_stream(stream);
  const PrepLayout pl = prep_layout(h->L, K);
  const char* pb = static_cast<const char*>(prep);
  const float lnr0 = (float)T.lo, inv_bw = (float)(nbands / (T.hi - T.lo));
  const float rmin = (float)exp((double)T.lo), rmax = (float)exp((double)T.hi);
  XT_REQUIRE(engine == 0 || engine == 1, "engine: 0 mma.sync, 1 tcgen05");
  int rc = radial_pass(T, h, prep, K, a_prior, c0, c1, band_use, nbands, xyzw, n, engine,
                       static_cast<float*>(workspace), st);
  if (rc) return rc;

  LearnArgs la{};
  la.T = Tf;
  la.GH = static_cast<const float*>(field_f32);
  la.CS = reinterpret_cast<const float*>(pb + pl.cs);
  la.R = static_cast<const float*>(workspace);
  la.rstride = r_stride(T.lmax);
  la.K = K;
  la.lmax = T.lmax;
  la.no_odd = no_odd;
  la.a_inv = (float)(1.0 / a_prior);
  la.rmin = rmin;
  la.rmax = rmax;
  la.lnr0 = lnr0;
  la.inv_bw = inv_bw;
  for (int b = 0; b < nbands; ++b) la.band_use[b] = band_use[b] != 0;
  la.nb = nbands;
  la.xyzw = reinterpret_cast<const float4*>(xyzw);
  la.n = n;
  la.out = reinterpret_cast<float4*>(out);
  la.prior_in_R = 0;
  const size_t sh = ((size_t)(T.lmax + 1) * (T.lmax + 1) * K + MLP_KMAX) * 4;
  if (T.lmax <= 4) return launch_learned_eval<4>(la, sh, st);
  if (T.lmax <= 6) return launch_learned_eval<6>(la, sh, st);
  return launch_learned_eval<7>(la, sh, st);
}

int xt_learned_radial_pass(void* sph, void* mlp, const void* prep, int K, double a_prior, double c0, double c1,
                           const int* band_use, int nbands, const float* xyzw, long long n, int engine, float* R,
                           void* stream) {
  SphTab<double> T;
  XT_REQUIRE(sph_tabs(sph, &T, nullptr), "NULL SL table handle");
  MlpHandle* h = nullptr;
  XT_REQUIRE(mlp_view(mlp, &h), "NULL network handle");
  XT_REQUIRE(T.cmap == 2 && h->L == T.lmax + 1 && h->nout == 2 * K && K <= T.nmax, "network / table / K mismatch");
  XT_REQUIRE(prep && band_use && xyzw && R && n >= 0, "NULL argument");
  XT_REQUIRE(nbands >= 1 && nbands <= MAX_BANDS, "need 1 <= nbands <= %d", MAX_BANDS);
  XT_REQUIRE(engine == 0 || engine == 1, "engine: 0 mma.sync, 1 tcgen05");
  XT_REQUIRE((reinterpret_cast<uintptr_t>(xyzw) & 15) == 0, "xyzw must be a 16-byte aligned float4 array");
  XT_REQUIRE(a_prior > 0.0, "prior scale must be positive");
  return radial_pass(T, h, prep, K, a_prior, c0, c1, band_use, nbands, xyzw, n, engine, R, as_stream(stream));
}

int xt_learned_status(void) {
  int* d = nullptr;
  int rc = tc_error_flag(&d);
  if (rc) return rc;
  int v = 0;
  XT_CUDA(cudaDeviceSynchronize());
  XT_CUDA(cudaMemcpy(&v, d, sizeof(int), cudaMemcpyDeviceToHost));
  if (v) {
    const int zero = 0;
    XT_CUDA(cudaMemcpy(d, &zero, sizeof(int), cudaMemcpyHostToDevice));
    set_error("learned basis on the tensor cores (network pass or training GEMM): an MMA completion wait timed out");
    return XT_ERR_DEVICE;
  }
  return XT_OK;
}

}  // extern "C"
