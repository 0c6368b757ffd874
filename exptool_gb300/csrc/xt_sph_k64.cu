// Spherical kernels instantiated for double arithmetic.
#include "xt_sph_kern.cuh"

namespace xt {
#define XT_INST(LC)                                                                                              \
  template void launch_sph_deposit<double, LC>(const SphTab<double>&, const double*, const double*, const double*,   \
                                            const double*, long long, int, double*, int, int, cudaStream_t);   \
  template void launch_sph_eval<double, LC>(const SphTab<double>&, const double*, int, const double*, const double*,     \
                                         const double*, long long, const SphEvalOpts&, double* const*, int,    \
                                         int, cudaStream_t);
XT_INST(4)
XT_INST(6)
XT_INST(8)
#undef XT_INST
}  // namespace xt
