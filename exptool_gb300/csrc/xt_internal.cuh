// Internal cross-file accessors of the table handles (not part of the C ABI).
#pragma once

#include "xt_cyl.cuh"
#include "xt_sph.cuh"

namespace xt {
bool sph_tabs(void* handle, SphTab<double>* d, SphTab<float>* f);
bool sph_efp(void* handle, const double** efp);   // ef/sqrt(ev) table [l][n][node]
bool cyl_tabs(void* handle, CylTab<double>* d, CylTab<float>* f);
}  // namespace xt
