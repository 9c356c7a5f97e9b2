// Kernels of the learned warm start (conditioned MLP, BF16 operands, FP32
// accumulation and master weights); see mlp.cu for the layouts.
#pragma once
#include <cuda_runtime.h>

namespace bcg {

enum { MLP_EPI_TANH = 0, MLP_EPI_DTANH = 1, MLP_EPI_LOSS = 2 };
constexpr int MLP_NFEAT = 128;  // input features per sample

cudaError_t mlp_gemm_nn(int epi, const void* a, const void* b, const float* bias, const void* yprev,
                        const float* target, void* out_bf, float* out_f32, float* loss_part, int m, int n, int k,
                        int nout, int m_valid, float gscale, cudaStream_t st);
cudaError_t mlp_gemm_tn(const void* a, const void* b, float* part, int m, int n1, int n2, int nsplit,
                        cudaStream_t st);
cudaError_t mlp_colsum(const void* dz, int m, int n, int nsplit, float* part, cudaStream_t st);
cudaError_t mlp_adam(const float* wpart, int nsplit, const float* bpart, int bsplit, int n1, int n2, float* w,
                     float* mw, float* vw, float* b, float* mb, float* vb, void* wbf, void* wtbf, float lr,
                     float beta1, float beta2, float eps, float* grad_out, cudaStream_t st);
cudaError_t mlp_cast_weights(const float* w, int n1, int n2, void* wbf, void* wtbf, cudaStream_t st);
cudaError_t mlp_features(const float* theta, const float* rho, int ncell, const float* params, int nset,
                         const float* targets, int nout, long long seed, int set, int m, int m_valid, void* x,
                         float* t, cudaStream_t st);
cudaError_t mlp_sum(const float* x, int n, float* out, cudaStream_t st);

}  // namespace bcg
