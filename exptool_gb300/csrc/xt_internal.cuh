// Internal cross-file accessors of the table handles (not part of the C ABI).
#pragma once

#include "xt_cyl.cuh"
#include "xt_sph.cuh"

namespace xt {
bool sph_tabs(void* handle, SphTab<double>* d, SphTab<float>* f);
bool cyl_tabs(void* handle, CylTab<double>* d, CylTab<float>* f);
}  // namespace xt
