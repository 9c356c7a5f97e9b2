// DNC5 residual and fused residual + JVP kernels for sm_103a.
//
// Reference: srcfv/prepro/flux_num_dnc5.f90 (primal), the Tapenade tangent
// srcfv/tangent/flux_num_dnc5_d.f90 (S = DK<K> here).
//
// GB300 note: the stencil is bound by the FP64 pipe, not by HBM, so every
// cell primitive, cell gradient and face flux is computed exactly once and
// parked in HBM scratch (L2-resident for the grid sizes of interest); the
// memory traffic this costs is far below the bandwidth roof.
#include "residual_impl.cuh"

namespace bcg {

void launch_primal_passes(const Ext& e, const Coef& c, const double* w, double* pr, double* gr, const double* nx,
                          const double* ny, const double* vol, cudaStream_t st) {
  const int B = 256;
  const GroupStride gs{0, 0};
  k_prim<double><<<(unsigned)((e.np + B - 1) / B), B, 0, st>>>(e, c, State<double>{w}, Scratch<double>{pr, e.np}, gs);
  if (c.k2 != 0.0)
    k_grad<double><<<(unsigned)((e.im * e.jm + B - 1) / B), B, 0, st>>>(e, c, Scratch<double>{pr, e.np},
                                                                        Scratch<double>{gr, e.np}, nx, ny, vol, gs);
}

size_t residual_scratch_doubles(int im, int jm, int gh, int ndir) {
  const Ext e = make_ext(im, jm, gh);
  const size_t nn = (size_t)(im + 1) * (jm + 1);
  return (size_t)(ndir + 1) * ((size_t)(F_NPRIM + S_NSENS + Q_NQ) * e.np + 10 * nn);
}

cudaError_t run_residual(const ResidualArgs& a, cudaStream_t st) {
  if (a.order != 0 && a.order != 5) return run_residual_scheme(a, st);
  switch (a.ndir) {
    case 0: return run_residual_t<double, 3>(a, st);
    case 1: return run_residual_t<DK<1>, 3>(a, st);
    case 2: return run_residual_t<DK<2>, 3>(a, st);
    case 4: return run_residual_t<DK<4>, 3>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace bcg
