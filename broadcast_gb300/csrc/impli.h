// Launch interface of the matrix-free implicit phase
// (srcfv/lhs/impli_matrix_free.F90:7 impli_matrix_free_2d).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>

namespace bcg {

struct ImpliArgs {
  int im, jm, gh, lmax;
  double dtcoef, cfl, gam, rgaz, prandtl, cv, cs, muref, tref, s_suth;
  const double* nx;   // (ni+1, nj+1, 2)
  const double* ny;
  const double* w;    // (ni, nj, 5) state with filled ghosts
  const double* dw;   // (ni, nj, 5) right-hand side (the residual), interior read
  const double* vol;  // (ni, nj)
  const double* volf; // (ni, nj, 2)
  double* dwi;        // (ni, nj, 5) increment; every ghost is zero on return
  double* scratch;    // impli_scratch_doubles(im, jm, gh) doubles
};

size_t impli_scratch_doubles(int im, int jm, int gh);
// the CTAs of the one thread-block cluster that runs the sweeps (16, or 8
// where the device cannot schedule a 16-CTA cluster)
int impli_cluster_size();
// the largest jm the sweep kernel takes (96 rows per CTA of the cluster)
int impli_max_rows();
cudaError_t run_impli(const ImpliArgs& a, cudaStream_t st);

}  // namespace bcg
