// Newton-Krylov linear solves: FP32 band LU factors kept on the device as
// preconditioners, FP64 CSR products and restarted FP64 GMRES (krylov.cu).
#pragma once
#include <cuda_runtime.h>

namespace bcg {

// FP32 band LU with partial pivoting of the row-equilibrated n x n CSR matrix
// (device arrays; perm optional, row/column k of A is factorised as perm[k]);
// *handle names the factor until band32_destroy.  Returns BCG_ERR_SINGULAR
// with *info = the first zero pivot (1-based) when the FP32 factor is singular.
int band32_factor(int n, const int* indptr, const int* indices, const double* data, const int* perm, int nb,
                  cudaStream_t st, long long* handle, int* info);
// x = M^-1 b with the factor (device FP64 vectors); synchronises st
int band32_solve(long long handle, const double* b, double* x, cudaStream_t st);
int band32_destroy(long long handle);
int band32_dims(long long handle, int* klku_nb);
// y = A x, or y = b - A x when b is given (FP64 CSR, device arrays)
int spmv(int n, const int* indptr, const int* indices, const double* data, const double* x, const double* b, double* y,
         cudaStream_t st);
// A x = b by restarted GMRES(restart), right-preconditioned by the factor,
// from x = 0 until ||b - A x|| <= rtol ||b|| or maxit iterations in total
int gmres_solve(long long handle, int n, const int* indptr, const int* indices, const double* data, const double* b,
                double* x, int restart, int maxit, double rtol, cudaStream_t st, int* iters, double* relres);

}  // namespace bcg
