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
  std::vector<JnArgs> joins;  // periodic joins applied to each tangent after the fills (wr = wd = the tangent)
  int withjn;               // 1: columns wrap periodically in i (computejacobianfromjv[_relaxed]_withjn)
  int nzone;                // 2: seeds in the two azimuthal zones i < imid, i >= imid (testvector_partial)
                            //    with computejacobianfromjv_relaxed_withjnandcheck's columns; else 1
  int imid;                 // first 0-based column of the second zone (a multiple of 7)
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
  // several operators from one pass over the seeds (nops > 0: op, the output
  // fields above and divide_by_vol are replaced by these; relaxed applies to
  // the residual tangent only)
  int nops;
  int ops[3];
  int divide_v[3];
  int* indptr_v[3];
  int* indices_v[3];
  double* data_v[3];
  long long capacity_v[3];
  long long* nnz_v[3];
};

// J(beta) = J - beta^2 Dzz + i beta Dz on the union pattern (biglobal.py:82);
// values: nbeta planes of nnz complex numbers (re, im interleaved)
struct CsrBetaArgs {
  int nrow;
  const int* j_p; const int* j_i; const double* j_v;
  const int* dz_p; const int* dz_i; const double* dz_v;
  const int* dzz_p; const int* dzz_i; const double* dzz_v;
  int nbeta;
  const double* betas;    // device, nbeta
  int* indptr;            // nrow + 1
  int* indices;           // capacity
  double* values;         // 2 * nbeta * capacity
  long long capacity;
  long long* nnz;         // host
  int* iscratch;          // csr_beta_iscratch_ints(nrow)
};
int run_csr_beta(const CsrBetaArgs& a, cudaStream_t st);
size_t csr_beta_iscratch_ints(int nrow);

size_t jacobian_scratch_doubles(int im, int jm, int gh, int nzone = 1, int nops = 1);
size_t jacobian_iscratch_ints(int im, int jm);
int run_jacobian(const JacobianArgs& a, cudaStream_t st);

}  // namespace bcg
