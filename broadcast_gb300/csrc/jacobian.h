// Batched colored Jacobian assembly (all seeds, CSR output).
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <vector>
#include "bc.h"
#include "dnc5.cuh"

namespace bcg {

struct JacobianArgs {
  int im, jm, gh;
  Phys phys;
  const double* w;          // state with its ghosts filled by the primal boundary chain
  const double* nx;
  const double* ny;
  const double* vol;
  const double* volf;
  std::vector<BcArgs> bcs;  // linearised boundary chain, in the drivers' order
  int op;                   // 0: residual tangent (Jacobian); SPAN_DZ / SPAN_DZZ: spanwise operators
  int relaxed;              // 1: coefdiag added on the diagonal (computejacobianfromjv_relaxed)
  const double* coefdiag;   // (im, jm)
  double mini;              // entries with |a| <= mini are dropped (remove_zero_jac)
  int divide_by_vol;        // 1: values divided by the row cell's volume (Jacvol)
  int* indptr;              // 5*im*jm + 1
  int* indices;             // capacity
  double* data;             // capacity
  long long capacity;
  long long* nnz;           // host: number of stored entries
  double* scratch;          // jacobian_scratch_doubles
  int* iscratch;            // jacobian_iscratch_ints
};

size_t jacobian_scratch_doubles(int im, int jm, int gh);
size_t jacobian_iscratch_ints(int im, int jm);
int run_jacobian(const JacobianArgs& a, cudaStream_t st);

}  // namespace bcg
