// Field-composition and leapfrog kernels instantiated for float force arithmetic.
#include "xt_orbit_kern.cuh"

namespace xt {
#define XT_INST(LC)                                                                                              \
  template void launch_fields_forces<float, LC>(const SphTab<float>&, const float*, const CylTab<float>&, const float*,     \
                                              const FieldOpts&, const double*, const double*, const double*,   \
                                              const double*, double, long long, double* const*, int, int,      \
                                              cudaStream_t);                                                   \
  template void launch_leapfrog<float, LC>(const SphTab<float>&, const float*, const CylTab<float>&, const float*,          \
                                         const FieldOpts&, const OrbitArgs&, int, int, cudaStream_t);
XT_INST(4)
XT_INST(6)
XT_INST(8)
#undef XT_INST
}  // namespace xt
