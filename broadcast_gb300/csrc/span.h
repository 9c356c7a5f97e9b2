// Launch interface of the spanwise operators Dz and Dzz.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include "dnc5.cuh"

namespace bcg {

enum SpanOp { SPAN_DZ = 1, SPAN_DZZ = 2 };

struct SpanArgs {
  int im, jm, gh;
  int op;               // SPAN_DZ (coeffs_5p_dz) or SPAN_DZZ (coeffs_5p_dz2)
  int ndir;             // 1, 2 or 4 directions per launch
  Phys phys;            // k2, k4 unused
  const double* w;      // base flow (ni, nj, 5)
  const double* wd;     // ndir stacked (ni, nj, 5) directions, stride dstride
  size_t dstride;
  const double* nx;     // (ni+1, nj+1, 2); Dz only
  const double* ny;
  const double* vol;    // (ni, nj); Dz only
  double* out;          // ndir stacked (ni, nj, 5), interior written, stride dstride
};

cudaError_t run_span(const SpanArgs& a, cudaStream_t st);

}  // namespace bcg
