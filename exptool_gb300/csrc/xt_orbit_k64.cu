// Field-composition and leapfrog kernels instantiated for double force arithmetic.
#include "xt_orbit_kern.cuh"

namespace xt {
#define XT_INST(LC)                                                                                              \
  template void launch_fields_forces<double, LC>(const SphTab<double>&, const double*, const CylTab<double>&, const double*,     \
                                              const FieldOpts&, const double*, const double*, const double*,   \
                                              const double*, double, long long, double* const*, int, int,      \
                                              cudaStream_t);                                                   \
  template void launch_leapfrog<double, LC>(const SphTab<double>&, const double*, const CylTab<double>&, const double*,          \
                                         const FieldOpts&, const OrbitArgs&, int, int, cudaStream_t);
XT_INST(4)
XT_INST(6)
XT_INST(8)
#undef XT_INST
}  // namespace xt
