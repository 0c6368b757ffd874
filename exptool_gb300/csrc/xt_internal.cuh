// Internal cross-file accessors of the table handles (not part of the C ABI).
#pragma once

#include "xt_cyl.cuh"
#include "xt_sph.cuh"

namespace xt {
bool sph_tabs(void* handle, SphTab<double>* d, SphTab<float>* f);
bool sph_efp(void* handle, const double** efp);   // ef/sqrt(ev) table [l][n][node]
bool sph_efp_df(void* handle, const float2** efp_df);   // the same as FP32 (hi, lo) pairs
bool cyl_tabs(void* handle, CylTab<double>* d, CylTab<float>* f);
// expcoef[s, row, n] = sum_node efp[l, n, node] G[s, row, node] for nsnap
// snapshot grids G (FP64, or double-float (hi, lo) pairs), in double-float
// from the split table efp_df (xt_batch.cu)
int launch_sph_contract_batched(const float2* efp_df, const double* G, int nsnap, int lmax, int nmax, int numr,
                                double* out, cudaStream_t st);
// exclusive scan of ncell <= 2^20 counts (xt_cyl.cu); tile_sum: 1024 ints
int launch_cell_scan(const int* hist, int* off, int* tile_sum, int ncell, cudaStream_t st);
int launch_sph_contract_batched(const float2* efp_df, const float2* G, int nsnap, int lmax, int nmax, int numr,
                                double* out, cudaStream_t st);
}  // namespace xt
