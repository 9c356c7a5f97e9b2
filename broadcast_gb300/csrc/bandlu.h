// Direct solve of a banded sparse system on the GPU (band LU with partial
// pivoting through cuSOLVER/cuBLAS on views of the band storage).
#pragma once
#include <cuda_runtime.h>

namespace bcg {

struct BandLuInfo {
  int kl, ku, nb, info;  // bandwidths found, block size, first zero pivot (1-based row) or 0
  long long ldab;        // leading dimension of the band storage
};

// x = A^-1 b for the n x n CSR matrix A (device arrays; duplicates summed);
// returns 0, 1 for a singular matrix (out->info = first zero pivot), -1 on
// another failure (band_lu_error() says which).  Synchronises the stream.
// q (optional, device): row and column k of A become row and column q[k] of
// the factorised matrix (a bandwidth-reducing order); must be a permutation.
int band_lu_solve(int n, const int* indptr, const int* indices, const double* data, const int* q, const double* b,
                  double* x, int nb, cudaStream_t st, BandLuInfo* out);
const char* band_lu_error();

}  // namespace bcg
