// Device calibration: the FP64 FMA throughput of the current GPU, the
// denominator of the FP64 roofline this stencil is bound by.
#include <cuda_runtime.h>
#include "runtime.h"

namespace {
__global__ void k_fp64_fma(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

extern "C" int bcg_fp64_peak_tflops(double* tflops) {
  using namespace bcg;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail_arg("fp64 peak: no CUDA device"), BCG_ERR_NODEV;
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail_cuda("fp64 peak: device query", e);
  const int B = 256, G = sms * 8, iters = 4096;
  double* out = (double*)pool_get(POOL_AUX, sizeof(double) * B * G);
  if (!out) return BCG_ERR_NOMEM;
  cudaStream_t st = current_stream();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0, st);
    k_fp64_fma<<<G, B, 0, st>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail_cuda("fp64 peak", e);
  *tflops = 2.0 * 8 * iters * (double)B * G / best / 1e9;
  return BCG_OK;
}
