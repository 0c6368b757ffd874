// Orbit frequencies: batched spectra of orbit signals with the peak search
// fused in, for exptool/orbits/frequencies.py:25-217.
//
// One CTA per signal (an orbit's column of a map).  The N-point discrete
// Fourier transform the reference takes with numpy.fft.fft is computed in
// double-float complex arithmetic on the FP32 pipe (GB300's FP64 pipe issues
// at a small fraction of the FP32 rate):
//  * N a power of two: one Stockham FFT of size M = N in shared memory,
//    radix-4 stages after at most one radix-2 stage (two ping-pong buffers,
//    natural-order output, no bit reversal);
//  * other N: Bluestein's chirp-z transform, X[k] = w[k] sum_n x[n] w[n]
//    conj(w[k - n]) with w[n] = exp(-i pi n^2 / N), as a circular convolution of
//    size M = 2^p >= 2N - 1 by two FFTs and the precomputed FFT of the chirp.
// Twiddles, chirp and its FFT come from the host in FP64 (angles reduced
// exactly in integers), split into FP32 pairs.  The spectrum stays in shared
// memory for the peak search:
//  * mode 0 (fundamental frequencies, frequencies.py:94-132): strict relative
//    maxima of |Re X| against `order` neighbours each side (indices clipped at
//    the ends), positive frequencies only, the three strongest;
//  * mode 1 (orbit frequencies, frequencies.py:135-217): the first index of
//    the largest |X| (compared as |X|^2), bin 0 set to zero on request.
// The caller maps indices to numpy.fft.fftfreq values.
#include <cfloat>

#include "xt_df.cuh"
#include "xt_internal.cuh"

namespace xt {

struct cdf {
  df re, im;
};

__device__ __forceinline__ cdf c_add(cdf a, cdf b) { return {df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ cdf c_sub(cdf a, cdf b) { return {df_sub(a.re, b.re), df_sub(a.im, b.im)}; }
__device__ __forceinline__ cdf c_mul(cdf a, cdf b) {
  return {df_sub(df_mul(a.re, b.re), df_mul(a.im, b.im)), df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
__device__ __forceinline__ cdf c_conj(cdf a) { return {a.re, df_neg(a.im)}; }
__device__ __forceinline__ cdf c_ld(const float4* p) {
  const float4 v = *p;
  return {{v.x, v.y}, {v.z, v.w}};
}
__device__ __forceinline__ void c_st(float4* p, cdf a) { *p = make_float4(a.re.h, a.re.l, a.im.h, a.im.l); }

__device__ __forceinline__ df df_absv(df a) { return a.h < 0.f ? df_neg(a) : a; }

// exp(-2 pi i t / m) for 0 <= t < m from the half table tw[t] (t < m / 2):
// W^t = -W^(t - m/2).
__device__ __forceinline__ cdf twiddle(const float4* __restrict__ tw, int t, int half) {
  cdf w = c_ld(tw + (t < half ? t : t - half));
  if (t >= half) {
    w.re = df_neg(w.re);
    w.im = df_neg(w.im);
  }
  return w;
}

// In-shared-memory Stockham FFT of size m (a power of two) from x, using y
// as the other buffer; returns the buffer holding the result (natural
// order).  Radix-4 stages (a leading radix-2 stage when log2 m is odd): a
// butterfly at offset j of sub-transform size ns reads x[j + r m/4], r < 4,
// multiplies by W_{4ns}^{r k} (k = j mod ns) and writes the four outputs of
// the 4-point DFT (W_4 = -i) to y[(j - k) 4 + k + r ns].  tw[t] =
// exp(-2 pi i t / m), t < m/2.  All threads of the CTA take part.
__device__ float4* fft_stockham(float4* x, float4* y, int m, const float4* __restrict__ tw) {
  const int half = m >> 1;
  int ns = 1;
  if ((31 - __clz(m)) & 1) {                   // radix-2 stage, ns = 1: no twiddles
    for (int j = threadIdx.x; j < half; j += blockDim.x) {
      const cdf v0 = c_ld(x + j), v1 = c_ld(x + j + half);
      c_st(y + 2 * j, c_add(v0, v1));
      c_st(y + 2 * j + 1, c_sub(v0, v1));
    }
    __syncthreads();
    float4* t = x;
    x = y;
    y = t;
    ns = 2;
  }
  const int q = m >> 2;
  for (; ns < m; ns <<= 2) {
    const int step = m / (4 * ns);               // W_{4 ns}^k = W_m^{k m / (4 ns)}
#pragma unroll 2
    for (int j = threadIdx.x; j < q; j += blockDim.x) {
      const int k = j & (ns - 1);
      const cdf a0 = c_ld(x + j);
      cdf a1 = c_ld(x + j + q), a2 = c_ld(x + j + 2 * q), a3 = c_ld(x + j + 3 * q);
      if (k) {
        a1 = c_mul(a1, twiddle(tw, k * step, half));
        a2 = c_mul(a2, twiddle(tw, 2 * k * step, half));
        a3 = c_mul(a3, twiddle(tw, 3 * k * step, half));
      }
      const cdf t0 = c_add(a0, a2), t1 = c_sub(a0, a2), t2 = c_add(a1, a3), d13 = c_sub(a1, a3);
      const cdf t3{d13.im, df_neg(d13.re)};      // -i (a1 - a3)
      const int d = ((j - k) << 2) + k;
      c_st(y + d, c_add(t0, t2));
      c_st(y + d + ns, c_add(t1, t3));
      c_st(y + d + 2 * ns, c_sub(t0, t2));
      c_st(y + d + 3 * ns, c_sub(t1, t3));
    }
    __syncthreads();
    float4* t = x;
    x = y;
    y = t;
  }
  return x;
}

struct SpecArgs {
  int mode, n, m, bluestein, order, zero_first, freq_sign;
  long long nsig, ld;
  const double *a, *b;       // signal s, sample t at a[t * ld + s] (+ i b[...] when b != NULL)
  const double* win;         // [n] window (numpy.hanning values) or NULL
  const float4 *tw, *chirp, *chirp_f;   // [m/2], [n], [m] complex df
  int* idx_out;              // [nsig][3]
  double* val_out;           // [nsig][3]
  double* spec_out;          // [nsig][n][2] or NULL
};

// numpy.fft.fftfreq(n, d)[k] > 0 with d of sign freq_sign
__device__ __forceinline__ bool positive_freq(int k, int n, int freq_sign) {
  const bool lowhalf = k >= 1 && k <= (n - 1) / 2;
  const bool highhalf = k >= (n + 1) / 2 && k < n;
  return freq_sign > 0 ? lowhalf : highhalf;
}

// Candidate order of the peak lists: larger value first, equal values by
// smaller index; index -1 marks an empty slot and sorts last.  Indices are
// distinct, so the order is total and the top three of a union do not depend
// on the order of the merges.
__device__ __forceinline__ bool cand_before(df v, int k, df w, int j) {
  if (k < 0) return false;
  if (j < 0) return true;
  return df_gt(v, w) || (!df_gt(w, v) && k < j);
}

// Insertion of (v, k) into a sorted three-entry list (fixed indices, so the
// list stays in registers).
__device__ __forceinline__ void insert3(df av[3], int ai[3], df v, int k) {
  if (!cand_before(v, k, av[2], ai[2])) return;
  av[2] = v;
  ai[2] = k;
  if (cand_before(av[2], ai[2], av[1], ai[1])) {
    const df tv = av[1];
    const int ti = ai[1];
    av[1] = av[2];
    ai[1] = ai[2];
    av[2] = tv;
    ai[2] = ti;
    if (cand_before(av[1], ai[1], av[0], ai[0])) {
      const df uv = av[0];
      const int ui = ai[0];
      av[0] = av[1];
      ai[0] = ai[1];
      av[1] = uv;
      ai[1] = ui;
    }
  }
}

// Every lane's sorted top-three list merged across the warp (butterfly
// shuffles: after five rounds each lane holds the warp's top three).
__device__ __forceinline__ void top3_warp(df v[3], int k[3]) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    df ov[3];
    int oi[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      ov[r].h = __shfl_xor_sync(0xffffffffu, v[r].h, off);
      ov[r].l = __shfl_xor_sync(0xffffffffu, v[r].l, off);
      oi[r] = __shfl_xor_sync(0xffffffffu, k[r], off);
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) insert3(v, k, ov[r], oi[r]);
  }
}

constexpr int SPEC_THREADS = 256;

__global__ void __launch_bounds__(SPEC_THREADS) k_orbit_spectra(SpecArgs a) {
  extern __shared__ float4 fsm[];
  __shared__ float r_hi[SPEC_THREADS / 32][3];
  __shared__ float r_lo[SPEC_THREADS / 32][3];
  __shared__ int r_idx[SPEC_THREADS / 32][3];
  float4* b0 = fsm;
  float4* b1 = fsm + a.m;
  const long long s = blockIdx.x;
  const int n = a.n, m = a.m;
  // the signal (windowed, chirped) into b0, zero-padded to m
  // (read-only global loads, free to be issued ahead of the shared-memory
  // stores of earlier samples)
#pragma unroll 4
  for (int t = threadIdx.x; t < m; t += blockDim.x) {
    cdf v{{0.f, 0.f}, {0.f, 0.f}};
    if (t < n) {
      v.re = df_from(__ldg(a.a + t * a.ld + s));
      v.im = df_from(a.b ? __ldg(a.b + t * a.ld + s) : 0.0);
      if (a.win) {
        const df wd = df_from(__ldg(a.win + t));
        v.re = df_mul(v.re, wd);
        v.im = df_mul(v.im, wd);
      }
      if (a.bluestein) v = c_mul(v, c_ld(a.chirp + t));
    }
    c_st(b0 + t, v);
  }
  __syncthreads();
  float4* X = fft_stockham(b0, b1, m, a.tw);
  if (a.bluestein) {
    // pointwise product with the chirp's transform, the inverse FFT as
    // conj(FFT(conj(.))) / m, then the output chirp
    float4* Y = X == b0 ? b1 : b0;
    for (int t = threadIdx.x; t < m; t += blockDim.x) c_st(X + t, c_conj(c_mul(c_ld(X + t), c_ld(a.chirp_f + t))));
    __syncthreads();
    X = fft_stockham(X, Y, m, a.tw);
    const float inv_m = 1.f / (float)m;                  // a power of two: exact
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      cdf v = c_conj(c_ld(X + t));
      v.re = {v.re.h * inv_m, v.re.l * inv_m};
      v.im = {v.im.h * inv_m, v.im.l * inv_m};
      c_st(X + t, c_mul(v, c_ld(a.chirp + t)));
    }
    __syncthreads();
  }
  if (a.spec_out)
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      const cdf v = c_ld(X + t);
      a.spec_out[(s * n + t) * 2] = df_to(v.re);
      a.spec_out[(s * n + t) * 2 + 1] = df_to(v.im);
    }
  // peak search: each thread keeps its best three (value as a df, index);
  // equal values keep the smaller index
  df bv[3];
  int bi[3];
  for (int q = 0; q < 3; ++q) {
    bv[q] = {-FLT_MAX, 0.f};
    bi[q] = -1;
  }
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const cdf c = c_ld(X + k);
    df v;
    bool cand = true;
    if (a.mode == 0) {
      v = df_absv(c.re);
      cand = positive_freq(k, n, a.freq_sign);
      for (int j = 1; cand && j <= a.order; ++j) {
        const int lo = k - j < 0 ? 0 : k - j, hi = k + j > n - 1 ? n - 1 : k + j;
        cand = df_gt(v, df_absv(c_ld(X + lo).re)) && df_gt(v, df_absv(c_ld(X + hi).re));
      }
    } else {
      // |X|^2 orders like |X|; the reference zeroes bin 0 and keeps it in the argmax
      v = (a.zero_first && k == 0) ? df{0.f, 0.f} : df_add(df_mul(c.re, c.re), df_mul(c.im, c.im));
    }
    if (cand) insert3(bv, bi, v, k);
  }
  // top three of the CTA: a shuffle tree inside each warp, then warp 0 merges
  // the warps' lists
  top3_warp(bv, bi);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
    for (int q = 0; q < 3; ++q) {
      r_hi[wid][q] = bv[q].h;
      r_lo[wid][q] = bv[q].l;
      r_idx[wid][q] = bi[q];
    }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    for (int q = 0; q < 3; ++q) {
      bv[q] = lane < nw ? df{r_hi[lane][q], r_lo[lane][q]} : df{-FLT_MAX, 0.f};
      bi[q] = lane < nw ? r_idx[lane][q] : -1;
    }
    top3_warp(bv, bi);
    if (lane == 0)
      for (int q = 0; q < 3; ++q) {
        a.idx_out[s * 3 + q] = bi[q];
        a.val_out[s * 3 + q] = bi[q] >= 0 ? df_to(bv[q]) : 0.0;
      }
  }
}

}  // namespace xt

using namespace xt;

extern "C" {

int xt_orbit_spectra(int mode, long long nsig, int n, const double* a, const double* b, long long ld,
                     const double* win, int order, int zero_first, int freq_sign, int m, const float* tw,
                     const float* chirp, const float* chirp_f, int* idx_out, double* val_out, double* spec_out,
                     void* stream) {
  XT_REQUIRE(mode == 0 || mode == 1, "mode must be 0 (fundamental) or 1 (peak)");
  XT_REQUIRE(nsig >= 0 && nsig < (1LL << 31) && n >= 1 && ld >= nsig, "bad signal sizes");
  XT_REQUIRE(m >= 2 && (m & (m - 1)) == 0 && m <= 4096, "transform size must be a power of two in [2, 4096], got %d",
             m);
  const bool blue = (n & (n - 1)) != 0;
  XT_REQUIRE(blue ? (m >= 2 * n - 1) : (m == n), "transform size %d does not fit signal length %d", m, n);
  XT_REQUIRE(order >= 0, "negative order");
  if (nsig == 0) return XT_OK;
  XT_REQUIRE(a && tw && idx_out && val_out, "NULL array");
  XT_REQUIRE(!blue || (chirp && chirp_f), "NULL chirp tables");
  XT_REQUIRE(((uintptr_t)tw & 15) == 0 && ((uintptr_t)chirp & 15) == 0 && ((uintptr_t)chirp_f & 15) == 0,
             "tables must be 16-byte aligned");
  SpecArgs A{mode, n, m, blue ? 1 : 0, order, zero_first ? 1 : 0, freq_sign >= 0 ? 1 : -1, nsig, ld, a, b, win,
             reinterpret_cast<const float4*>(tw), reinterpret_cast<const float4*>(chirp),
             reinterpret_cast<const float4*>(chirp_f), idx_out, val_out, spec_out};
  const size_t smem = 2 * (size_t)m * sizeof(float4);
  static size_t attr = 0;
  if (smem > 48 * 1024 && smem > attr) {
    XT_CUDA(cudaFuncSetAttribute(k_orbit_spectra, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = smem;
  }
  k_orbit_spectra<<<(unsigned)nsig, SPEC_THREADS, smem, as_stream(stream)>>>(A);
  XT_CHECK_LAUNCH("k_orbit_spectra");
  return XT_OK;
}

}  // extern "C"
