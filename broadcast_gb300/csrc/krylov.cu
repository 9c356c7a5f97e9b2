// Newton-Krylov linear solves on the GPU: FP64 GMRES on the assembled Newton
// matrix, right-preconditioned by an FP32 band LU of it.
//
// The reference solves each Newton system J dw = R with a sparse direct LU
// (PETSc/MUMPS, BROADCAST_npz.py:1146-1158, misc/PETSc_func.py:137-152).  An
// FP64 band LU does the same on the GPU (bandlu.cu), but its cost grows as
// n kl^2 and GB300's FP64 rate is ~1/60 of its FP32 rate: on the 512 x 256
// O-mesh (kl = 7715) one FP64 factorisation takes minutes.  Here the same
// banded LU (LAPACK's blocked dgbtrf algorithm: cuSOLVER getrf panels, cuBLAS
// trsm/gemm trailing updates, one panel of lookahead on a second stream) runs
// in FP32 on the row-equilibrated matrix (each row scaled by 1/max|a_rj|), and
// serves as the preconditioner M of restarted GMRES whose matrix products,
// orthogonalisation and solution stay in FP64:
//   A M^-1 u = b,  x = M^-1 u,  M^-1 v = P^T U^-1 L^-1 P S v
// (S the row scaling, P the bandwidth-reducing permutation).  The converged
// dw satisfies the FP64 system to GMRES's tolerance, so the Newton iteration
// converges as with the direct solve; an FP32 factor of a neighbouring matrix
// (the previous Newton step, a nearby base flow) remains a good preconditioner,
// so factorisations can be reused.
//
// Orthogonalisation: classical Gram-Schmidt with one re-orthogonalisation
// (two cuBLAS gemv per pass over the basis), Givens rotations of the
// Hessenberg column on the host.
#include <cublas_v2.h>
#include <cusolverDn.h>
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>
#include "krylov.h"
#include "runtime.h"

namespace bcg {

namespace {

__global__ void k_bandwidth32(int n, const int* __restrict__ indptr, const int* __restrict__ indices,
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

// row scaling s[r] = 1 / max_j |a_rj| (1 for an empty row) and the scaled
// entries in FP32 at their permuted band positions
__global__ void k_fill_band32(int n, const int* __restrict__ indptr, const int* __restrict__ indices,
                              const double* __restrict__ data, const int* __restrict__ q, double* __restrict__ rs,
                              float* __restrict__ ab, long long ldab, int U) {
  const int r0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (r0 >= n) return;
  double mx = 0.0;
  for (int p = indptr[r0]; p < indptr[r0 + 1]; ++p) mx = fmax(mx, fabs(data[p]));
  const double s = mx > 0.0 ? 1.0 / mx : 1.0;
  rs[r0] = s;
  const long long r = q ? q[r0] : r0;
  for (int p = indptr[r0]; p < indptr[r0 + 1]; ++p) {
    const long long c = q ? q[indices[p]] : indices[p];
    ab[U + r - c + c * ldab] += (float)(s * data[p]);
  }
}

__global__ void k_laswp32(float* __restrict__ d, long long ld, int ncol, const int* __restrict__ ipiv, int jb) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncol) return;
  float* col = d + (long long)c * ld;
  for (int t = 0; t < jb; ++t) {
    const int p = ipiv[t] - 1;
    if (p != t) { const float x = col[t]; col[t] = col[p]; col[p] = x; }
  }
}

__global__ void k_note_info32(const int* __restrict__ info, int* __restrict__ first, int j0) {
  if (threadIdx.x == 0 && blockIdx.x == 0 && *first == 0 && *info > 0) *first = j0 + *info;
}

// gather index of each block's row swaps: after the swaps ipiv[0..jb) of a
// panel, row t of its m-row window holds the former row perm[t]
__global__ void k_block_perms(int n, int nb, int kl, const int* __restrict__ ipiv, const long long* __restrict__ off,
                              int* __restrict__ perm) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j0 = k * nb;
  if (j0 >= n) return;
  const int jb = min(nb, n - j0), m = min(kl + jb, n - j0);
  int* p = perm + off[k];
  for (int t = 0; t < m; ++t) p[t] = t;
  for (int t = 0; t < jb; ++t) {
    const int q = ipiv[j0 + t] - 1;
    if (q != t) { const int x = p[t]; p[t] = p[q]; p[q] = x; }
  }
}

// identity matrices of size jb x jb (ld nb) for every block
__global__ void k_identity_blocks(int n, int nb, float* __restrict__ a) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)n * nb) return;
  const int k = (int)(e / ((long long)nb * nb));
  const long long r = e - (long long)k * nb * nb;
  const int i = (int)(r % nb), j = (int)(r / nb);
  a[e] = (i == j && k * nb + i < n) ? 1.0f : 0.0f;
}

// pointers of one apply (read by the captured graph's first and last kernels)
struct ApplyArgs { const double* v; double* z; };

__global__ void k_scale_in_args(int n, const int* __restrict__ q, const double* __restrict__ s,
                                const ApplyArgs* __restrict__ args, float* __restrict__ xf) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  xf[q ? q[k] : k] = (float)(s[k] * args->v[k]);
}

__global__ void k_permute_out_args(int n, const int* __restrict__ q, const float* __restrict__ xf,
                                   const ApplyArgs* __restrict__ args) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  args->z[k] = (double)xf[q ? q[k] : k];
}

// a panel's row swaps on its m-row window of w, as one gather through shared
// memory (one CTA)
__global__ void __launch_bounds__(1024) k_gather_window(float* __restrict__ w, const int* __restrict__ perm, int m) {
  extern __shared__ float seg[];
  for (int t = threadIdx.x; t < m; t += blockDim.x) seg[t] = w[t];
  __syncthreads();
  for (int t = threadIdx.x; t < m; t += blockDim.x) w[t] = seg[perm[t]];
}

// y = A x (or y = b - A x with b given), FP64 CSR, one warp per row
__global__ void __launch_bounds__(256) k_spmv(int n, const int* __restrict__ indptr, const int* __restrict__ indices,
                                              const double* __restrict__ data, const double* __restrict__ x,
                                              const double* __restrict__ b, double* __restrict__ y) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  double acc = 0.0;
  for (int p = indptr[row] + lane; p < indptr[row + 1]; p += 32) acc = fma(data[p], __ldg(x + indices[p]), acc);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) y[row] = b ? b[row] - acc : acc;
}

struct Band32 {
  int n = 0, kl = 0, ku = 0, nb = 0, nblk = 0;
  long long ldab = 0, ldd = 0;
  float* ab = nullptr;
  int* ipiv = nullptr;
  int* q = nullptr;
  double* rs = nullptr;
  float* xf = nullptr;        // forward working vector (swapped and updated right-hand side)
  float* yf = nullptr;        // forward result, then the backward right-hand side
  float* zf = nullptr;        // backward result
  float* linv = nullptr;      // per block: L_kk^-1 (nb x nb, unit lower)
  float* uinv = nullptr;      // per block: U_kk^-1 (nb x nb, upper)
  int* perms = nullptr;       // per block: gather index of its row swaps (m_k entries)
  std::vector<long long> poff;  // per block: offset of its gather index
  ApplyArgs* args = nullptr;  // device copy of the current apply's pointers
  cudaStream_t gs = nullptr;  // capture stream
  cudaGraphExec_t graph = nullptr;
  int dev = 0;
};

struct KHandles {
  cublasHandle_t blas = nullptr, blas_b = nullptr;
  cusolverDnHandle_t sol = nullptr;
  cudaStream_t sb = nullptr;
};
std::mutex g_mu;
std::map<int, KHandles> g_kh;                 // per device
std::map<long long, Band32*> g_factors;
long long g_next = 1;

int handles_for(int dev, KHandles** out) {
  KHandles& h = g_kh[dev];
  if (!h.blas && cublasCreate(&h.blas) != CUBLAS_STATUS_SUCCESS) return fail_arg("cublasCreate failed");
  if (!h.blas_b && cublasCreate(&h.blas_b) != CUBLAS_STATUS_SUCCESS) return fail_arg("cublasCreate failed");
  if (!h.sol && cusolverDnCreate(&h.sol) != CUSOLVER_STATUS_SUCCESS) return fail_arg("cusolverDnCreate failed");
  if (!h.sb && cudaStreamCreateWithFlags(&h.sb, cudaStreamNonBlocking) != cudaSuccess)
    return fail_cuda("krylov: stream", cudaGetLastError());
  *out = &h;
  return BCG_OK;
}

void free_band(Band32* f) {
  if (!f) return;
  if (f->graph) cudaGraphExecDestroy(f->graph);
  if (f->gs) cudaStreamDestroy(f->gs);
  cudaFree(f->ab); cudaFree(f->ipiv); cudaFree(f->q); cudaFree(f->rs); cudaFree(f->xf);
  cudaFree(f->yf); cudaFree(f->zf); cudaFree(f->linv); cudaFree(f->uinv); cudaFree(f->perms); cudaFree(f->args);
  delete f;
}

// the launches of one apply of M^-1 (pointers from f->args) on stream st:
// scale and permute in; per block forward: the panel's swaps (one CTA), then
// L_kk^-1 and L21 products (cuBLAS gemv); per block backward: U12 and U_kk^-1
// products; permute out
int band32_launch(const Band32* f, KHandles* h, cudaStream_t st) {
  const int n = f->n, nb = f->nb, kl = f->kl, ku = f->ku;
  const long long ldd = f->ldd;
  const int U = kl + ku + nb;
  float* dv = f->ab + U;
  auto D = [&](long long i, long long j) { return dv + i + j * ldd; };
  const float one = 1.0f, zero = 0.0f, mone = -1.0f;
  cublasSetStream(h->blas, st);
  cublasSetPointerMode(h->blas, CUBLAS_POINTER_MODE_HOST);
  const int B = 256;
  k_scale_in_args<<<(n + B - 1) / B, B, 0, st>>>(n, f->q, f->rs, f->args, f->xf);
  for (int k = 0; k < f->nblk; ++k) {
    const int j0 = k * nb, jb = std::min(nb, n - j0), m = std::min(kl + jb, n - j0);
    k_gather_window<<<1, 1024, (size_t)m * sizeof(float), st>>>(f->xf + j0, f->perms + f->poff[k], m);
    if (cublasSgemv(h->blas, CUBLAS_OP_N, jb, jb, &one, f->linv + (size_t)k * nb * nb, nb, f->xf + j0, 1, &zero,
                    f->yf + j0, 1) != CUBLAS_STATUS_SUCCESS) return fail_arg("band32: gemv failed");
    if (m > jb && cublasSgemv(h->blas, CUBLAS_OP_N, m - jb, jb, &mone, D(j0 + jb, j0), (int)ldd, f->yf + j0, 1, &one,
                              f->xf + j0 + jb, 1) != CUBLAS_STATUS_SUCCESS) return fail_arg("band32: gemv failed");
  }
  for (int k = f->nblk - 1; k >= 0; --k) {
    const int j0 = k * nb, jb = std::min(nb, n - j0), ncol = std::min(n - j0 - jb, kl + ku);
    if (ncol > 0 && cublasSgemv(h->blas, CUBLAS_OP_N, jb, ncol, &mone, D(j0, j0 + jb), (int)ldd, f->zf + j0 + jb, 1,
                                &one, f->yf + j0, 1) != CUBLAS_STATUS_SUCCESS) return fail_arg("band32: gemv failed");
    if (cublasSgemv(h->blas, CUBLAS_OP_N, jb, jb, &one, f->uinv + (size_t)k * nb * nb, nb, f->yf + j0, 1, &zero,
                    f->zf + j0, 1) != CUBLAS_STATUS_SUCCESS) return fail_arg("band32: gemv failed");
  }
  k_permute_out_args<<<(n + B - 1) / B, B, 0, st>>>(n, f->q, f->zf, f->args);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? BCG_OK : fail_cuda("band32 apply", e);
}

// M^-1 v into z (device FP64 vectors) on stream st: the launches replayed from
// a CUDA graph captured on the factor's first apply (or queued directly when
// capture is not possible)
int band32_apply(Band32* f, KHandles* h, const double* v, double* z, cudaStream_t st) {
  const ApplyArgs a{v, z};
  cudaError_t e = cudaMemcpyAsync(f->args, &a, sizeof(a), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return fail_cuda("band32 apply: arguments", e);
  if (!f->graph && !f->gs) {
    if (cudaStreamCreateWithFlags(&f->gs, cudaStreamNonBlocking) == cudaSuccess) {
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(f->gs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const int rc = band32_launch(f, h, f->gs);
        const cudaError_t ec = cudaStreamEndCapture(f->gs, &g);
        if (rc == BCG_OK && ec == cudaSuccess && g && cudaGraphInstantiate(&f->graph, g, 0) != cudaSuccess)
          f->graph = nullptr;
        if (g) cudaGraphDestroy(g);
      }
      cudaGetLastError();  // a failed capture falls back to direct launches
    }
    cublasSetStream(h->blas, st);  // the handle is shared with the caller's stream work
  }
  if (f->graph) {
    e = cudaGraphLaunch(f->graph, st);
    return e == cudaSuccess ? BCG_OK : fail_cuda("band32 apply: graph launch", e);
  }
  return band32_launch(f, h, st);
}

Band32* factor_of(long long hnd) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_factors.find(hnd);
  return it == g_factors.end() ? nullptr : it->second;
}

}  // namespace

int band32_factor(int n, const int* indptr, const int* indices, const double* data, const int* perm, int nb,
                  cudaStream_t st, long long* handle, int* info) {
  if (n < 1 || !indptr || !indices || !data || !handle) return fail_arg("band32_factor: bad arguments");
  int dev = 0;
  cudaGetDevice(&dev);
  KHandles* h = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    const int rc = handles_for(dev, &h);
    if (rc) return rc;
  }
  Band32* f = new Band32();
  f->n = n; f->dev = dev;
  int* d_klku = nullptr;
  int* d_info = nullptr;
  float* work = nullptr;
  cudaEvent_t ev_a = nullptr, ev_b = nullptr;
  int rc = BCG_OK;
  auto bad = [&](int code) { rc = code; };
  do {
    const int B = 256;
    if (cudaMalloc(&d_klku, 4 * sizeof(int)) != cudaSuccess) { bad(fail_arg("band32: allocation failed")); break; }
    cudaMemsetAsync(d_klku, 0, 4 * sizeof(int), st);
    if (perm) {
      if (cudaMalloc(&f->q, (size_t)n * sizeof(int)) != cudaSuccess) { bad(fail_arg("band32: allocation failed")); break; }
      cudaMemcpyAsync(f->q, perm, (size_t)n * sizeof(int), cudaMemcpyDefault, st);
    }
    k_bandwidth32<<<(n + B - 1) / B, B, 0, st>>>(n, indptr, indices, f->q, d_klku);
    int klku[2] = {0, 0};
    if (cudaMemcpyAsync(klku, d_klku, 2 * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) { bad(fail_cuda("band32: bandwidth", cudaGetLastError())); break; }
    const int kl = klku[0], ku = klku[1];
    nb = std::max(1, std::min(std::min(nb, 1024), n));
    const int L = kl + nb, U = kl + ku + nb;
    f->kl = kl; f->ku = ku; f->nb = nb;
    // the forward solve holds a panel's window (kl + nb rows) in shared memory
    const size_t seg = (size_t)(kl + nb) * sizeof(float);
    if (seg > 227 * 1024) { bad(fail_arg("band32: lower bandwidth too large (kl + nb > 58112)")); break; }
    if (seg > 48 * 1024 &&
        cudaFuncSetAttribute(k_gather_window, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)seg) != cudaSuccess) {
      bad(fail_cuda("band32: shared memory", cudaGetLastError()));
      break;
    }
    f->ldab = (long long)L + U + 1;
    f->ldd = f->ldab - 1;
    const size_t bytes = (size_t)f->ldab * (size_t)n * sizeof(float);
    if (cudaMalloc(&f->ab, bytes) != cudaSuccess) { cudaGetLastError(); bad(fail_arg("band32: band storage allocation failed")); break; }
    if (cudaMalloc(&f->ipiv, (size_t)n * sizeof(int)) != cudaSuccess || cudaMalloc(&f->rs, (size_t)n * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&f->xf, (size_t)n * sizeof(float)) != cudaSuccess || cudaMalloc(&d_info, sizeof(int)) != cudaSuccess) {
      cudaGetLastError();
      bad(fail_arg("band32: allocation failed"));
      break;
    }
    cudaMemsetAsync(f->ab, 0, bytes, st);
    k_fill_band32<<<(n + B - 1) / B, B, 0, st>>>(n, indptr, indices, data, f->q, f->rs, f->ab, f->ldab, U);
    float* dv = f->ab + U;
    const long long ldd = f->ldd;
    auto D = [&](long long i, long long j) { return dv + i + j * ldd; };
    cublasSetStream(h->blas, st);
    cublasSetStream(h->blas_b, h->sb);
    cusolverDnSetStream(h->sol, st);
    cublasSetPointerMode(h->blas, CUBLAS_POINTER_MODE_HOST);
    cublasSetPointerMode(h->blas_b, CUBLAS_POINTER_MODE_HOST);
    int lwork = 0;
    if (cusolverDnSgetrf_bufferSize(h->sol, std::min(kl + nb, n), nb, D(0, 0), (int)ldd, &lwork) != CUSOLVER_STATUS_SUCCESS) {
      bad(fail_arg("band32: getrf buffer size failed"));
      break;
    }
    if (cudaMalloc(&work, (size_t)std::max(lwork, 1) * sizeof(float)) != cudaSuccess) { bad(fail_arg("band32: allocation failed")); break; }
    if (cudaEventCreateWithFlags(&ev_a, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev_b, cudaEventDisableTiming) != cudaSuccess) { bad(fail_arg("band32: events")); break; }
    const float one = 1.0f, mone = -1.0f;
    auto update = [&](cublasHandle_t hb, cudaStream_t s, int j0, int jb, int m, int c0, int nc) -> bool {
      if (nc <= 0) return true;
      k_laswp32<<<(nc + 127) / 128, 128, 0, s>>>(D(j0, c0), ldd, nc, f->ipiv + j0, jb);
      if (cublasStrsm(hb, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_UNIT, jb, nc, &one,
                      D(j0, j0), (int)ldd, D(j0, c0), (int)ldd) != CUBLAS_STATUS_SUCCESS) { bad(fail_arg("band32: trsm failed")); return false; }
      if (m > jb && cublasSgemm(hb, CUBLAS_OP_N, CUBLAS_OP_N, m - jb, nc, jb, &mone, D(j0 + jb, j0), (int)ldd,
                                D(j0, c0), (int)ldd, &one, D(j0 + jb, c0), (int)ldd) != CUBLAS_STATUS_SUCCESS) {
        bad(fail_arg("band32: gemm failed"));
        return false;
      }
      return true;
    };
    for (int j0 = 0; j0 < n && rc == BCG_OK; j0 += nb) {
      const int jb = std::min(nb, n - j0);
      const int m = std::min(kl + jb, n - j0);
      if (cusolverDnSgetrf(h->sol, m, jb, D(j0, j0), (int)ldd, work, f->ipiv + j0, d_info) != CUSOLVER_STATUS_SUCCESS) {
        bad(fail_arg("band32: getrf failed"));
        break;
      }
      k_note_info32<<<1, 1, 0, st>>>(d_info, d_klku + 2, j0);
      const int ncol = std::min(n - j0 - jb, kl + ku);
      const int nnext = std::min(ncol, nb);
      cudaEventRecord(ev_a, st);
      cudaStreamWaitEvent(h->sb, ev_a, 0);
      if (!update(h->blas_b, h->sb, j0, jb, m, j0 + jb + nnext, ncol - nnext)) break;
      if (j0 > 0) cudaStreamWaitEvent(st, ev_b, 0);
      if (!update(h->blas, st, j0, jb, m, j0 + jb, nnext)) break;
      cudaEventRecord(ev_b, h->sb);
    }
    cudaEventRecord(ev_b, h->sb);
    cudaStreamWaitEvent(st, ev_b, 0);
    if (rc) break;
    int first = 0;
    if (cudaMemcpyAsync(&first, d_klku + 2, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) { bad(fail_cuda("band32: factorisation", cudaGetLastError())); break; }
    if (info) *info = first;
    if (first) { bad(fail_arg("band32: singular matrix (zero pivot)")); rc = BCG_ERR_SINGULAR; break; }
    // for the solves: each block's swaps as a gather index, the inverses of
    // the diagonal blocks of L and U, work vectors
    f->nblk = (n + nb - 1) / nb;
    f->poff.assign(f->nblk + 1, 0);
    for (int k = 0; k < f->nblk; ++k) {
      const int j0 = k * nb, jb = std::min(nb, n - j0);
      f->poff[k + 1] = f->poff[k] + std::min(kl + jb, n - j0);
    }
    const size_t inv = (size_t)f->nblk * nb * nb;
    long long* d_off = nullptr;
    if (cudaMalloc(&f->perms, (size_t)f->poff.back() * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&d_off, (size_t)(f->nblk + 1) * sizeof(long long)) != cudaSuccess ||
        cudaMalloc(&f->linv, inv * sizeof(float)) != cudaSuccess || cudaMalloc(&f->uinv, inv * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&f->yf, (size_t)n * sizeof(float)) != cudaSuccess || cudaMalloc(&f->zf, (size_t)n * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&f->args, sizeof(ApplyArgs)) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(d_off);
      bad(fail_arg("band32: allocation of the solve data failed"));
      break;
    }
    cudaMemcpyAsync(d_off, f->poff.data(), (size_t)(f->nblk + 1) * sizeof(long long), cudaMemcpyHostToDevice, st);
    k_block_perms<<<(f->nblk + 127) / 128, 128, 0, st>>>(n, nb, kl, f->ipiv, d_off, f->perms);
    const long long nall = (long long)f->nblk * nb * nb;
    k_identity_blocks<<<(unsigned)((nall + 255) / 256), 256, 0, st>>>(f->nblk * nb, nb, f->linv);
    k_identity_blocks<<<(unsigned)((nall + 255) / 256), 256, 0, st>>>(f->nblk * nb, nb, f->uinv);
    for (int k = 0; k < f->nblk && rc == BCG_OK; ++k) {
      const int j0 = k * nb, jb = std::min(nb, n - j0);
      float* li = f->linv + (size_t)k * nb * nb;
      float* ui = f->uinv + (size_t)k * nb * nb;
      if (cublasStrsm(h->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_LOWER, CUBLAS_OP_N, CUBLAS_DIAG_UNIT, jb, jb, &one,
                      D(j0, j0), (int)ldd, li, nb) != CUBLAS_STATUS_SUCCESS ||
          cublasStrsm(h->blas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, jb, jb, &one,
                      D(j0, j0), (int)ldd, ui, nb) != CUBLAS_STATUS_SUCCESS) bad(fail_arg("band32: block inverse failed"));
    }
    cudaStreamSynchronize(st);
    cudaFree(d_off);
    if (rc) break;
  } while (false);
  cudaStreamSynchronize(st);
  if (ev_a) cudaEventDestroy(ev_a);
  if (ev_b) cudaEventDestroy(ev_b);
  cudaFree(work);
  cudaFree(d_info);
  cudaFree(d_klku);
  if (rc != BCG_OK) { free_band(f); return rc; }
  std::lock_guard<std::mutex> lk(g_mu);
  *handle = g_next++;
  g_factors[*handle] = f;
  return BCG_OK;
}

int band32_solve(long long hnd, const double* b, double* x, cudaStream_t st) {
  Band32* f = factor_of(hnd);
  if (!f) return fail_arg("band32: unknown factor");
  KHandles* h = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    const int rc = handles_for(f->dev, &h);
    if (rc) return rc;
  }
  const int rc = band32_apply(f, h, b, x, st);
  if (rc) return rc;
  const cudaError_t e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? BCG_OK : fail_cuda("band32 solve", e);
}

int band32_destroy(long long hnd) {
  Band32* f = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_factors.find(hnd);
    if (it == g_factors.end()) return fail_arg("band32: unknown factor");
    f = it->second;
    g_factors.erase(it);
  }
  cudaDeviceSynchronize();
  free_band(f);
  return BCG_OK;
}

int band32_dims(long long hnd, int* klku_nb) {
  Band32* f = factor_of(hnd);
  if (!f || !klku_nb) return fail_arg("band32: unknown factor");
  klku_nb[0] = f->kl; klku_nb[1] = f->ku; klku_nb[2] = f->nb;
  return BCG_OK;
}

int spmv(int n, const int* indptr, const int* indices, const double* data, const double* x, const double* b, double* y,
         cudaStream_t st) {
  const int B = 256;
  k_spmv<<<(unsigned)(((long long)n * 32 + B - 1) / B), B, 0, st>>>(n, indptr, indices, data, x, b, y);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? BCG_OK : fail_cuda("spmv", e);
}

int gmres_solve(long long hnd, int n, const int* indptr, const int* indices, const double* data, const double* b,
                double* x, int restart, int maxit, double rtol, cudaStream_t st, int* iters, double* relres) {
  Band32* f = factor_of(hnd);
  if (!f) return fail_arg("gmres: unknown preconditioner factor");
  if (f->n != n) return fail_arg("gmres: the factor's size differs from the system's");
  if (restart < 1 || maxit < 1) return fail_arg("gmres: restart and maxit must be >= 1");
  KHandles* h = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    const int rc = handles_for(f->dev, &h);
    if (rc) return rc;
  }
  const int m = restart;
  double *V = nullptr, *w = nullptr, *z = nullptr, *hcol = nullptr;
  const size_t nn = (size_t)n;
  if (cudaMalloc(&V, nn * (m + 1) * sizeof(double)) != cudaSuccess || cudaMalloc(&w, nn * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&z, nn * sizeof(double)) != cudaSuccess || cudaMalloc(&hcol, (size_t)(2 * m + 2) * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(V); cudaFree(w); cudaFree(z); cudaFree(hcol);
    return fail_arg("gmres: allocation failed"), BCG_ERR_NOMEM;
  }
  cublasHandle_t bl = h->blas;
  cublasSetStream(bl, st);
  cublasSetPointerMode(bl, CUBLAS_POINTER_MODE_HOST);
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), hh(m + 1), hh2(m + 1), y(m);
  int rc = BCG_OK, it = 0;
  double bnorm = 0.0, res = 0.0;
  const double one = 1.0, zero = 0.0, mone = -1.0;
  auto ok = [&](cublasStatus_t s) { if (s != CUBLAS_STATUS_SUCCESS) { rc = fail_arg("gmres: cuBLAS call failed"); return false; } return true; };
  do {
    if (!ok(cublasDnrm2(bl, n, b, 1, &bnorm))) break;
    if (bnorm == 0.0) { cudaMemsetAsync(x, 0, nn * sizeof(double), st); res = 0.0; break; }
    cudaMemsetAsync(x, 0, nn * sizeof(double), st);
    bool done = false;
    while (!done && rc == BCG_OK) {
      // r = b - A x into V_0
      if ((rc = spmv(n, indptr, indices, data, x, b, V, st))) break;
      double beta = 0.0;
      if (!ok(cublasDnrm2(bl, n, V, 1, &beta))) break;
      res = beta / bnorm;
      if (res <= rtol || it >= maxit) { done = true; break; }
      const double ib = 1.0 / beta;
      if (!ok(cublasDscal(bl, n, &ib, V, 1))) break;
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int j = 0;
      for (; j < m && it < maxit; ++j, ++it) {
        double* vj = V + nn * j;
        if ((rc = band32_apply(f, h, vj, z, st))) break;
        if ((rc = spmv(n, indptr, indices, data, z, nullptr, w, st))) break;
        // classical Gram-Schmidt, twice
        if (!ok(cublasDgemv(bl, CUBLAS_OP_T, n, j + 1, &one, V, n, w, 1, &zero, hcol, 1))) break;
        if (!ok(cublasDgemv(bl, CUBLAS_OP_N, n, j + 1, &mone, V, n, hcol, 1, &one, w, 1))) break;
        if (!ok(cublasDgemv(bl, CUBLAS_OP_T, n, j + 1, &one, V, n, w, 1, &zero, hcol + m + 1, 1))) break;
        if (!ok(cublasDgemv(bl, CUBLAS_OP_N, n, j + 1, &mone, V, n, hcol + m + 1, 1, &one, w, 1))) break;
        if (cudaMemcpyAsync(hh.data(), hcol, (j + 1) * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(hh2.data(), hcol + m + 1, (j + 1) * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) {
          rc = fail_cuda("gmres: copy", cudaGetLastError());
          break;
        }
        double hn = 0.0;
        if (!ok(cublasDnrm2(bl, n, w, 1, &hn))) break;  // synchronises the stream
        for (int i = 0; i <= j; ++i) H[(size_t)i + (size_t)j * (m + 1)] = hh[i] + hh2[i];
        H[(size_t)(j + 1) + (size_t)j * (m + 1)] = hn;
        if (hn > 0.0) {
          const double ihn = 1.0 / hn;
          if (!ok(cublasDcopy(bl, n, w, 1, V + nn * (j + 1), 1))) break;
          if (!ok(cublasDscal(bl, n, &ihn, V + nn * (j + 1), 1))) break;
        }
        // Givens rotations of the new column
        for (int i = 0; i < j; ++i) {
          double& a = H[(size_t)i + (size_t)j * (m + 1)];
          double& c2 = H[(size_t)(i + 1) + (size_t)j * (m + 1)];
          const double t = cs[i] * a + sn[i] * c2;
          c2 = -sn[i] * a + cs[i] * c2;
          a = t;
        }
        double& a = H[(size_t)j + (size_t)j * (m + 1)];
        double& c2 = H[(size_t)(j + 1) + (size_t)j * (m + 1)];
        const double r = std::hypot(a, c2);
        cs[j] = r > 0.0 ? a / r : 1.0;
        sn[j] = r > 0.0 ? c2 / r : 0.0;
        a = r;
        c2 = 0.0;
        g[j + 1] = -sn[j] * g[j];
        g[j] = cs[j] * g[j];
        res = std::fabs(g[j + 1]) / bnorm;
        if (res <= rtol || hn == 0.0) { ++j; ++it; break; }
      }
      if (rc) break;
      // y = H^-1 g (upper triangular j x j), u = V y, x += M^-1 u
      const int k = j;
      for (int i = k - 1; i >= 0; --i) {
        double s = g[i];
        for (int l = i + 1; l < k; ++l) s -= H[(size_t)i + (size_t)l * (m + 1)] * y[l];
        y[i] = s / H[(size_t)i + (size_t)i * (m + 1)];
      }
      if (k > 0) {
        if (cudaMemcpyAsync(hcol, y.data(), k * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess) {
          rc = fail_cuda("gmres: copy", cudaGetLastError());
          break;
        }
        if (!ok(cublasDgemv(bl, CUBLAS_OP_N, n, k, &one, V, n, hcol, 1, &zero, w, 1))) break;
        if ((rc = band32_apply(f, h, w, z, st))) break;
        if (!ok(cublasDaxpy(bl, n, &one, z, 1, x, 1))) break;
      }
      // the loop head recomputes the true residual and stops or restarts
    }
  } while (false);
  cudaStreamSynchronize(st);
  cudaFree(V); cudaFree(w); cudaFree(z); cudaFree(hcol);
  if (iters) *iters = it;
  if (relres) *relres = res;
  return rc;
}

}  // namespace bcg
