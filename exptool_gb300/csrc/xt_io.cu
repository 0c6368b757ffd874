// Particle-record de-interleaving for the snapshot readers (EXP PSP / SPL
// files, exptool/io/psp_io.py:196-230 and spl_io.py:235-270 read them through
// a NumPy structured memmap): packed records of rec_bytes bytes, every field
// 4 or 8 bytes at a 4-byte offset, become one array per field.
//
// A block stages kRecTile records at a time in shared memory with 16-byte
// loads of the contiguous record bytes (the records may sit in page-locked
// host memory and are then read over the host link once, coalesced), and
// writes each field as a coalesced column.  Columns may likewise be device
// or page-locked host memory.
#include <algorithm>
#include <cstring>

#include "xt_internal.cuh"

namespace xt {

constexpr int kRecTile = 128;        // records per staged tile
constexpr int kMaxCols = 32;
constexpr int kMaxRecBytes = 384;    // 128 * 384 B = 48 KB of staging

struct RecCols {
  int ncol;
  int off[kMaxCols];
  int kind[kMaxCols];
  void* out[kMaxCols];
};

__global__ void __launch_bounds__(256) k_records_to_columns(const unsigned char* __restrict__ rec, long long n,
                                                            int rec_bytes, RecCols C) {
  extern __shared__ unsigned int stage[];                 // kRecTile * rec_bytes / 4 words
  const int wpr = rec_bytes >> 2;                          // words per record
  const long long ntile = (n + kRecTile - 1) / kRecTile;
  for (long long t = blockIdx.x; t < ntile; t += gridDim.x) {
    const long long r0 = t * kRecTile;
    const int nrec = (int)min((long long)kRecTile, n - r0);
    const int nwords = nrec * wpr;
    const unsigned char* src = rec + r0 * rec_bytes;
    // r0 * rec_bytes is a multiple of 16 (kRecTile * rec_bytes is), so the
    // tile is 16-byte aligned whenever `rec` is
    const bool vec = ((reinterpret_cast<uintptr_t>(src) & 15) == 0);
    if (vec) {
      const int nv = nwords >> 2;
      const uint4* s4 = reinterpret_cast<const uint4*>(src);
      for (int i = threadIdx.x; i < nv; i += blockDim.x) {
        const uint4 v = s4[i];
        stage[4 * i] = v.x;
        stage[4 * i + 1] = v.y;
        stage[4 * i + 2] = v.z;
        stage[4 * i + 3] = v.w;
      }
      for (int i = 4 * nv + threadIdx.x; i < nwords; i += blockDim.x)
        stage[i] = reinterpret_cast<const unsigned int*>(src)[i];
    } else {
      for (int i = threadIdx.x; i < nwords; i += blockDim.x) stage[i] = reinterpret_cast<const unsigned int*>(src)[i];
    }
    __syncthreads();
    for (int task = threadIdx.x; task < nrec * C.ncol; task += blockDim.x) {
      const int r = task % nrec, c = task / nrec;
      const unsigned int* w = stage + r * wpr + (C.off[c] >> 2);
      const long long i = r0 + r;
      switch (C.kind[c]) {
        case XT_COL_F32:
          static_cast<float*>(C.out[c])[i] = __uint_as_float(w[0]);
          break;
        case XT_COL_F32_TO_F64:
          static_cast<double*>(C.out[c])[i] = (double)__uint_as_float(w[0]);
          break;
        case XT_COL_I32:
          static_cast<int*>(C.out[c])[i] = (int)w[0];
          break;
        case XT_COL_F64:
          static_cast<double*>(C.out[c])[i] = __hiloint2double((int)w[1], (int)w[0]);
          break;
        default:   // XT_COL_I64
          static_cast<long long*>(C.out[c])[i] = (long long)(((unsigned long long)w[1] << 32) | w[0]);
          break;
      }
    }
    __syncthreads();
  }
}

}  // namespace xt

using namespace xt;

extern "C" {

int xt_records_to_columns(const void* records, long long n, int rec_bytes, int ncol, const int* col_off,
                          const int* col_kind, void* const* outs, void* stream) {
  XT_REQUIRE(n >= 0, "negative record count");
  if (n == 0) return XT_OK;
  XT_REQUIRE(records && col_off && col_kind && outs, "NULL argument");
  XT_REQUIRE(rec_bytes > 0 && rec_bytes % 4 == 0 && rec_bytes <= kMaxRecBytes,
             "record size %d must be a positive multiple of 4, at most %d", rec_bytes, kMaxRecBytes);
  XT_REQUIRE(ncol > 0 && ncol <= kMaxCols, "column count %d not in [1, %d]", ncol, kMaxCols);
  XT_REQUIRE(pointer_access(records) != XT_PTR_INACCESSIBLE, "records are host memory the device cannot address");
  RecCols C;
  memset(&C, 0, sizeof(C));
  C.ncol = ncol;
  for (int c = 0; c < ncol; ++c) {
    const int k = col_kind[c];
    XT_REQUIRE(k >= XT_COL_F32 && k <= XT_COL_F32_TO_F64, "column %d: bad kind %d", c, k);
    const int size = (k == XT_COL_F64 || k == XT_COL_I64) ? 8 : 4;
    XT_REQUIRE(col_off[c] >= 0 && col_off[c] % 4 == 0 && col_off[c] + size <= rec_bytes,
               "column %d: field at byte %d (size %d) outside the %d-byte record or not 4-byte aligned", c,
               col_off[c], size, rec_bytes);
    XT_REQUIRE(outs[c], "column %d: NULL output", c);
    XT_REQUIRE(pointer_access(outs[c]) != XT_PTR_INACCESSIBLE, "column %d: host memory the device cannot address",
               c);
    C.off[c] = col_off[c];
    C.kind[c] = k;
    C.out[c] = outs[c];
  }
  const size_t smem = (size_t)kRecTile * rec_bytes;
  if (smem > 48 * 1024)
    XT_CUDA(cudaFuncSetAttribute(k_records_to_columns, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const long long ntile = (n + kRecTile - 1) / kRecTile;
  const int grid = (int)std::min<long long>(ntile, (long long)resident_blocks_per_sm((const void*)k_records_to_columns,
                                                                                      256, smem) * sm_count());
  k_records_to_columns<<<grid, 256, smem, as_stream(stream)>>>(static_cast<const unsigned char*>(records), n,
                                                                rec_bytes, C);
  XT_CHECK_LAUNCH("k_records_to_columns");
  return XT_OK;
}

}  // extern "C"
