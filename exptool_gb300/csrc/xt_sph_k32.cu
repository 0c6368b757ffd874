// Spherical kernels instantiated for float arithmetic.
#include "xt_sph_kern.cuh"

namespace xt {
#define XT_INST(LC)                                                                                              \
  template void launch_sph_deposit<float, LC>(const SphTab<float>&, const double*, const double*, const double*,   \
                                            const double*, long long, int, double*, int, int, cudaStream_t);   \
  template void launch_sph_eval<float, LC>(const SphTab<float>&, const float*, int, const double*, const double*,     \
                                         const double*, long long, const SphEvalOpts&, double* const*, int,    \
                                         int, cudaStream_t);
XT_INST(4)
XT_INST(6)
XT_INST(8)
#undef XT_INST
}  // namespace xt
