// Direct sparse solve of the Newton system J dw = R on the GPU (the linear
// solve of the SER Newton iteration, BROADCAST_npz.py:1146-1158, where the
// reference factorises with PETSc/MUMPS on the host).
//
// The Jacobian rows are ordered (i, j, e) with i slowest, so every entry lies
// within kl = ku = 5 jm gh + 5 gh + 4 of the diagonal (the stencil reaches gh
// cells in i and j): a band of width ~15 jm.  The factorisation is LAPACK's
// blocked band LU with partial pivoting (dgbtrf's algorithm), run as dense
// library calls on views of the band storage:
//   band storage with lower bandwidth L = kl + nb and upper bandwidth
//   U = kl + ku + nb (ldab = L + U + 1), column-major, element (i, j) at
//   ab[U + i - j + j ldab] = ab[U + i + j (ldab - 1)], so any block within
//   the window is an ordinary dense matrix with leading dimension ldab - 1;
//   the extra nb rows above and below hold the panel's zero corner and the
//   pivoting fill-in (rows moved up by at most kl bring kl more columns);
//   per block column of nb: cuSOLVER getrf of the (kl + nb) x nb panel,
//   the panel's row swaps applied to its kl + ku trailing columns, cuBLAS
//   trsm for U12 and gemm for A22 -= L21 U12 (the flops: 2 n kl (kl + ku)).
// The solve applies each block's pivots, then L11^-1 and -L21 (forward), and
// U12, U11^-1 backwards, as dgbtrs does with the per-column pivots.
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <algorithm>
#include <cstdio>
#include "bandlu.h"

namespace bcg {
namespace {

// q: optional reordering, row/column k of A is row/column q[k] of the
// factorised matrix (null: the identity)
__global__ void k_bandwidth(int n, const int* __restrict__ indptr, const int* __restrict__ indices,
                            const int* __restrict__ q, int* klku) {
  const int r0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (r0 >= n) return;
  const int r = q ? q[r0] : r0;
  int lo = 0, hi = 0;
  for (int p = indptr[r0]; p < indptr[r0 + 1]; ++p) {
    const int c = q ? q[indices[p]] : indices[p];
    lo = max(lo, r - c);
    hi = max(hi, c - r);
  }
  atomicMax(klku, lo);
  atomicMax(klku + 1, hi);
}

__global__ void k_fill_band(int n, const int* __restrict__ indptr, const int* __restrict__ indices,
                            const double* __restrict__ data, const int* __restrict__ q, double* __restrict__ ab,
                            long long ldab, int U) {
  const int r0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (r0 >= n) return;
  const long long r = q ? q[r0] : r0;
  for (int p = indptr[r0]; p < indptr[r0 + 1]; ++p) {
    const long long c = q ? q[indices[p]] : indices[p];
    ab[U + r - c + c * ldab] += data[p];  // duplicates add, as a COO -> CSR conversion does
  }
}

// y[q[k]] = x[k] (forward) or y[k] = x[q[k]] (back)
__global__ void k_permute(int n, const int* __restrict__ q, const double* __restrict__ x, double* __restrict__ y,
                          int back) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  if (back) y[k] = x[q[k]]; else y[q[k]] = x[k];
}

// row swaps of one panel (pivots ipiv[0..jb), 1-based within the panel) on
// ncol columns of the dense view d (leading dimension ld); one thread per column
__global__ void k_laswp(double* __restrict__ d, long long ld, int ncol, const int* __restrict__ ipiv, int jb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncol) return;
  double* col = d + (long long)c * ld;
  for (int t = 0; t < jb; ++t) {
    const int p = ipiv[t] - 1;
    if (p != t) { const double x = col[t]; col[t] = col[p]; col[p] = x; }
  }
}

// keep the first zero pivot over all panels (getrf's info is per panel)
__global__ void k_note_info(const int* __restrict__ info, int* __restrict__ first, int j0) {
  if (threadIdx.x == 0 && blockIdx.x == 0 && *first == 0 && *info > 0) *first = j0 + *info;
}

// the same swaps on a vector (one thread: the swaps are sequential)
__global__ void k_swap_vec(double* __restrict__ b, const int* __restrict__ ipiv, int jb) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int t = 0; t < jb; ++t) {
    const int p = ipiv[t] - 1;
    if (p != t) { const double x = b[t]; b[t] = b[p]; b[p] = x; }
  }
}

struct Handles {
  cublasHandle_t blas = nullptr;    // on the caller's stream (panel path)
  cublasHandle_t blas_b = nullptr;  // on the trailing-update stream
  cusolverDnHandle_t sol = nullptr;
  cudaStream_t sb = nullptr;        // trailing-update stream
};
Handles g_h;

const char* g_err = "";

bool handles() {
  if (!g_h.blas && cublasCreate(&g_h.blas) != CUBLAS_STATUS_SUCCESS) { g_err = "cublasCreate failed"; return false; }
  if (!g_h.blas_b && cublasCreate(&g_h.blas_b) != CUBLAS_STATUS_SUCCESS) { g_err = "cublasCreate failed"; return false; }
  if (!g_h.sol && cusolverDnCreate(&g_h.sol) != CUSOLVER_STATUS_SUCCESS) { g_err = "cusolverDnCreate failed"; return false; }
  if (!g_h.sb && cudaStreamCreateWithFlags(&g_h.sb, cudaStreamNonBlocking) != cudaSuccess) {
    g_err = "stream creation failed";
    return false;
  }
  return true;
}

}  // namespace

const char* band_lu_error() { return g_err; }

int band_lu_solve(int n, const int* indptr, const int* indices, const double* data, const int* q, const double* b,
                  double* x, int nb, cudaStream_t st, BandLuInfo* out) {
  g_err = "";
  if (n < 1) { g_err = "empty system"; return -1; }
  if (!handles()) return -1;
  cublasSetStream(g_h.blas, st);
  cublasSetStream(g_h.blas_b, g_h.sb);
  cusolverDnSetStream(g_h.sol, st);
  cublasSetPointerMode(g_h.blas, CUBLAS_POINTER_MODE_HOST);
  cublasSetPointerMode(g_h.blas_b, CUBLAS_POINTER_MODE_HOST);
  cudaEvent_t ev_a = nullptr, ev_b = nullptr;  // panel done (stream st), trailing update done (stream sb)
  int* d_klku = nullptr;
  int* d_ipiv = nullptr;
  int* d_info = nullptr;
  double* ab = nullptr;
  double* work = nullptr;
  double* xq = nullptr;  // the solution in the factorised order
  int rc = 0;
  auto fail = [&](const char* m) { g_err = m; rc = -1; };
  do {
    if (cudaMalloc(&d_klku, 4 * sizeof(int)) != cudaSuccess) { fail("allocation failed"); break; }
    cudaMemsetAsync(d_klku, 0, 4 * sizeof(int), st);
    const int B = 256;
    k_bandwidth<<<(n + B - 1) / B, B, 0, st>>>(n, indptr, indices, q, d_klku);
    int klku[2] = {0, 0};
    if (cudaMemcpyAsync(klku, d_klku, 2 * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) { fail("bandwidth pass failed"); break; }
    const int kl = klku[0], ku = klku[1];
    nb = std::max(1, std::min(nb, n));
    const int L = kl + nb, U = kl + ku + nb;
    const long long ldab = (long long)L + U + 1, ldd = ldab - 1;
    if (out) { out->kl = kl; out->ku = ku; out->ldab = ldab; out->nb = nb; }
    const size_t bytes = (size_t)ldab * (size_t)n * sizeof(double);
    if (cudaMalloc(&ab, bytes) != cudaSuccess) { cudaGetLastError(); fail("band storage allocation failed"); break; }
    if (cudaMalloc(&d_ipiv, (size_t)n * sizeof(int)) != cudaSuccess) { fail("allocation failed"); break; }
    if (cudaMalloc(&d_info, sizeof(int)) != cudaSuccess) { fail("allocation failed"); break; }
    cudaMemsetAsync(ab, 0, bytes, st);
    k_fill_band<<<(n + B - 1) / B, B, 0, st>>>(n, indptr, indices, data, q, ab, ldab, U);
    double* d0 = ab + U;  // dense view: D(i, j) = d0[i + j * ldd]
    auto D = [&](long long i, long long j) { return d0 + i + j * ldd; };
    int lwork = 0;
    if (cusolverDnDgetrf_bufferSize(g_h.sol, std::min(kl + nb, n), nb, D(0, 0), (int)ldd, &lwork) !=
        CUSOLVER_STATUS_SUCCESS) { fail("getrf buffer size failed"); break; }
    if (cudaMalloc(&work, (size_t)std::max(lwork, 1) * sizeof(double)) != cudaSuccess) { fail("allocation failed"); break; }
    // factorisation, with a lookahead of one panel: on the caller's stream the
    // panel is factorised and the NEXT panel's columns are updated (swaps,
    // trsm, gemm), on the second stream the rest of the trailing columns; the
    // next panel's factorisation then overlaps this step's large trailing
    // gemm.  The operations and their operands are those of the plain
    // right-looking order, split over disjoint column sets.
    if (cudaEventCreateWithFlags(&ev_a, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev_b, cudaEventDisableTiming) != cudaSuccess) { fail("event creation failed"); break; }
    int first_singular = 0;
    const double one = 1.0, mone = -1.0;
    // the swaps, trsm and gemm of panel (j0, jb, m) on columns [c0, c0 + nc)
    auto update = [&](cublasHandle_t h, cudaStream_t s, int j0, int jb, int m, int c0, int nc) -> bool {
      if (nc <= 0) return true;
      k_laswp<<<(nc + 127) / 128, 128, 0, s>>>(D(j0, c0), ldd, nc, d_ipiv + j0, jb);
      if (cublasDtrsm(h, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_UNIT, jb, nc, &one,
                      D(j0, j0), (int)ldd, D(j0, c0), (int)ldd) != CUBLAS_STATUS_SUCCESS) { fail("trsm failed"); return false; }
      if (m > jb && cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, m - jb, nc, jb, &mone, D(j0 + jb, j0), (int)ldd,
                                D(j0, c0), (int)ldd, &one, D(j0 + jb, c0), (int)ldd) != CUBLAS_STATUS_SUCCESS) {
        fail("gemm failed");
        return false;
      }
      return true;
    };
    for (int j0 = 0; j0 < n && rc == 0; j0 += nb) {
      const int jb = std::min(nb, n - j0);
      const int m = std::min(kl + jb, n - j0);
      // panel j0 has all its updates: from the previous step's lookahead (this stream)
      if (cusolverDnDgetrf(g_h.sol, m, jb, D(j0, j0), (int)ldd, work, d_ipiv + j0, d_info) != CUSOLVER_STATUS_SUCCESS) {
        fail("getrf failed");
        break;
      }
      k_note_info<<<1, 1, 0, st>>>(d_info, d_klku + 2, j0);
      const int ncol = std::min(n - j0 - jb, kl + ku);
      const int nnext = std::min(ncol, nb);  // the next panel's columns
      // the rest of the trailing columns waits for this panel and runs on the second stream
      cudaEventRecord(ev_a, st);
      cudaStreamWaitEvent(g_h.sb, ev_a, 0);
      if (!update(g_h.blas_b, g_h.sb, j0, jb, m, j0 + jb + nnext, ncol - nnext)) break;
      // the next panel's columns were last updated by the previous step's rest
      // (recorded in ev_b before this step's rest was queued)
      if (j0 > 0) cudaStreamWaitEvent(st, ev_b, 0);
      if (!update(g_h.blas, st, j0, jb, m, j0 + jb, nnext)) break;
      cudaEventRecord(ev_b, g_h.sb);
    }
    if (rc == 0) {  // join the second stream
      cudaEventRecord(ev_b, g_h.sb);
      cudaStreamWaitEvent(st, ev_b, 0);
    }
    if (rc) break;
    if (cudaMemcpyAsync(&first_singular, d_klku + 2, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) { fail("factorisation failed"); break; }
    if (first_singular) {
      g_err = "singular matrix";
      if (out) out->info = first_singular;
      rc = 1;
      break;
    }
    // solve: x = b (reordered), then forward (pivots, L) and backward (U)
    if (q) {
      if (cudaMalloc(&xq, (size_t)n * sizeof(double)) != cudaSuccess) { fail("allocation failed"); break; }
      k_permute<<<(n + B - 1) / B, B, 0, st>>>(n, q, b, xq, 0);
    } else if (cudaMemcpyAsync(x, b, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
      fail("copy failed");
      break;
    }
    double* const xf = q ? xq : x;
    for (int j0 = 0; j0 < n && rc == 0; j0 += nb) {
      const int jb = std::min(nb, n - j0);
      const int m = std::min(kl + jb, n - j0);
      k_swap_vec<<<1, 1, 0, st>>>(xf + j0, d_ipiv + j0, jb);
      if (cublasDtrsv(g_h.blas, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_UNIT, jb, D(j0, j0), (int)ldd, xf + j0,
                      1) != CUBLAS_STATUS_SUCCESS) { fail("trsv failed"); break; }
      if (m > jb && cublasDgemv(g_h.blas, CUBLAS_OP_N, m - jb, jb, &mone, D(j0 + jb, j0), (int)ldd, xf + j0, 1, &one,
                                xf + j0 + jb, 1) != CUBLAS_STATUS_SUCCESS) { fail("gemv failed"); break; }
    }
    if (rc) break;
    const int nblk = (n + nb - 1) / nb;
    for (int k = nblk - 1; k >= 0 && rc == 0; --k) {
      const int j0 = k * nb;
      const int jb = std::min(nb, n - j0);
      const int ncol = std::min(n - j0 - jb, kl + ku);
      if (ncol > 0 && cublasDgemv(g_h.blas, CUBLAS_OP_N, jb, ncol, &mone, D(j0, j0 + jb), (int)ldd, xf + j0 + jb, 1, &one,
                                  xf + j0, 1) != CUBLAS_STATUS_SUCCESS) { fail("gemv failed"); break; }
      if (cublasDtrsv(g_h.blas, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, jb, D(j0, j0), (int)ldd,
                      xf + j0, 1) != CUBLAS_STATUS_SUCCESS) { fail("trsv failed"); break; }
    }
    if (q) k_permute<<<(n + B - 1) / B, B, 0, st>>>(n, q, xq, x, 1);
    if (out) out->info = 0;
  } while (false);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess && rc == 0) { g_err = cudaGetErrorString(e); rc = -1; }
  if (ev_a) cudaEventDestroy(ev_a);
  if (ev_b) cudaEventDestroy(ev_b);
  cudaFree(xq);
  cudaFree(work);
  cudaFree(d_info);
  cudaFree(d_ipiv);
  cudaFree(ab);
  cudaFree(d_klku);
  return rc;
}

}  // namespace bcg
