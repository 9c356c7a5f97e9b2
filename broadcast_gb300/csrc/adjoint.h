// Launch interface of the DNC5 adjoint (VJP) kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include "dnc5.cuh"

namespace bcg {

struct AdjointArgs {
  int im, jm, gh;
  Phys phys;
  const double* w;      // (ni, nj, 5)
  const double* nx;
  const double* ny;
  const double* vol;
  const double* volf;
  double* rb;           // residub (ni, nj, 5): interior read, then zeroed
  double* wb;           // (ni, nj, 5): overwritten on every padded cell
  double* scratch;      // adjoint_scratch_doubles(im, jm, gh) doubles
  int nowall;           // 1: flux_num_dnc5_nowall_2d_b (centred rows everywhere, no wall face)
  int ncot;             // cotangents in this call (0 or 1: one); rb and wb hold ncot blocks
  size_t cstride;       // doubles between consecutive cotangents' rb / wb blocks (0: 5 * padded cells)
};

// scratch of one call: primitives and gradients once, then per cotangent its
// gathered adjoints and face records
size_t adjoint_scratch_doubles(int im, int jm, int gh, int ncot = 1);
size_t adjoint_cotangent_doubles(int im, int jm, int gh);
cudaError_t run_adjoint(const AdjointArgs& a, cudaStream_t st);

}  // namespace bcg
