// Colored-Jacobian seeding/indexing and residual-norm kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>

namespace bcg {

// Modes of the COO fill; each follows one routine of misc/ComputeJacobian.f90.
enum JacMode {
  JAC_PLAIN = 0,           // computejacobianfromjv                 (:292-355)
  JAC_RELAXED = 1,         // computejacobianfromjv_relaxed         (:503-570)
  JAC_RELAXED_WITHJN = 2,  // computejacobianfromjv_relaxed_withjn  (:847-926)
  JAC_WITHJN = 3,          // computejacobianfromjv_withjn          (:929-999)
  JAC_DZ = 4,              // computejacobianfromdz                 (:708-779)
  JAC_CHECK = 5,           // computejacobianfromjv_relaxed_withjnandcheck (:1095-1204)
};

struct JacArgs {
  int mode, m, l, k, gh, im, jm, n;
  double mini;
  const double* resd;       // (ni, nj, 5) padded
  const double* coefdiag;   // (im, jm) or null
  double* jac;              // 5*im*jm slots of this seed (already offset)
  int* ia;
  int* ja;
};
cudaError_t launch_computejacobian(const JacArgs& a, cudaStream_t st);
// offset of the slots of seed (m,l,k[,n]) in the reference's COO arrays
long long jac_slot_base(int mode, int m, int l, int k, int gh, int im, int jm, int n);

cudaError_t launch_testvector(double* wd, int m, int l, int k, int gh, int im, int jm, int istart, int iend,
                              int jstart, int jend, bool partial, cudaStream_t st);

// norms of the interior of a padded (ni, nj, 5) array
enum NormKind { NORM_L2 = 0, NORM_L2INF = 1, NORM_MAX = 2 };
cudaError_t launch_norm(int kind, const double* rhs, int im, int jm, int gh, double* out /*device, 15 doubles*/,
                        double* partial /*device scratch*/, int npartial, cudaStream_t st);
int norm_partial_blocks(int im, int jm);

}  // namespace bcg
