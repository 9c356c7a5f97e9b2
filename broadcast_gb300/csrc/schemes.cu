// Residual and single-direction tangent of the DNC schemes of order 3, 7 and 9
// (srcfv/rhs/flux_num_dnc{3,7,9}.F90, the _nowall forms and their Tapenade
// tangents srcfv/tangent/flux_num_dnc{3,7,9}[_nowall]_d.f90): the DNC5 passes
// with R = 2, 4, 5 point pairs.  A separate translation unit, so that it
// compiles in parallel with the DNC5 kernels.
#include "residual_impl.cuh"

namespace bcg {

template <int R>
static cudaError_t run_order(const ResidualArgs& a, cudaStream_t st) {
  switch (a.ndir) {
    case 0: return run_residual_t<double, R>(a, st);
    case 1: return run_residual_t<DK<1>, R>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t run_residual_scheme(const ResidualArgs& a, cudaStream_t st) {
  if (a.ngroup > 1 || a.gh < dnc_pairs(a.order)) return cudaErrorInvalidValue;
  switch (a.order) {
    case 3: return run_order<2>(a, st);
    case 7: return run_order<4>(a, st);
    case 9: return run_order<5>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace bcg
