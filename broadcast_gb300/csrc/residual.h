// Launch interface of the DNC5 residual / fused residual + JVP kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include "dnc5.cuh"

namespace bcg {

struct ResidualArgs {
  int im, jm, gh;
  int ndir;              // 0: residual only; K: residual + K tangent directions
  Phys phys;
  const double* w;       // (ni, nj, 5)
  const double* wd;      // K stacked (ni, nj, 5) tangent states, stride dstride
  size_t dstride;        // doubles between tangent directions (>= 5*ni*nj)
  const double* nx;      // (ni+1, nj+1, 2)
  const double* ny;
  const double* vol;     // (ni, nj)
  const double* volf;    // (ni, nj, 2)
  double* res;           // (ni, nj, 5), interior written; may be null when ndir > 0
  double* resd;          // K stacked (ni, nj, 5), interior written
  double* scratch;       // ngroup * residual_scratch_doubles(im, jm, gh, ndir) doubles
  int nowall;            // 1: flux_num_dnc5_nowall_2d (centred rows everywhere, no wall face)
  int ngroup;            // 0 or 1: one group; G > 1 (ndir > 0): G groups of ndir directions in one launch,
                         // group g reading wd + g*ndir*dstride and writing resd + g*ndir*dstride
  int order;             // DNC scheme order: 0 or 5 (DNC5); 3, 7 or 9 (ndir 0 or 1; gh >= (order+1)/2)
  int rect;              // 1: the grid is rectilinear (face_rectilinear_*); DNC5 takes the face kernel
                         // without the products with the zero metric components
};

// Whether every i-face normal of the padded node set has ny = 0 and every
// j-face normal nx = 0 exactly (the faces the residual reads): host arrays,
// or device arrays (queued on st and waited for; false on an error).
bool face_rectilinear_host(const double* nx, const double* ny, int im, int jm, int gh);
bool face_rectilinear_device(const double* nx, const double* ny, int im, int jm, int gh, cudaStream_t st);
// the same, host or device arrays alike; device results that are false are
// remembered per (nx, ny, im, jm, gh) so that repeated calls on a curvilinear
// grid's resident metrics skip the check (a remembered false only costs speed),
// and a stream that is being captured into a graph gets false (no wait)
bool face_rectilinear(const double* nx, const double* ny, int im, int jm, int gh, cudaStream_t st);

size_t residual_scratch_doubles(int im, int jm, int gh, int ndir);
// primitives (and, when k2 != 0, gradients) of the primal state into scratch
// fields laid out as F_* and G_* planes of np doubles
void launch_primal_passes(const Ext& e, const Coef& c, const double* w, double* pr, double* gr, const double* nx,
                          const double* ny, const double* vol, cudaStream_t st);
cudaError_t run_residual(const ResidualArgs& a, cudaStream_t st);
// the DNC3, DNC7 and DNC9 schemes (a.order 3, 7, 9; ndir 0 or 1), schemes.cu
cudaError_t run_residual_scheme(const ResidualArgs& a, cudaStream_t st);

}  // namespace bcg
