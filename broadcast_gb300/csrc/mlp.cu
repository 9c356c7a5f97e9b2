// Learned warm start: the kernels that train and run the conditioned MLP
// mapping (Re, Mach) and a cell's position on the O-mesh to the converged
// base flow at that cell.  BF16 operands, FP32 accumulation on the tensor
// cores (mma.sync m16n8k16, operands staged through shared memory by
// cp.async and read with ldmatrix), FP32 master weights and Adam moments.
//
// Layouts (row-major, all device memory):
//   activations  X [M x K] bf16 (one row per sample), K a multiple of 64
//   weights      W [N x K] bf16 (one row per output), and its transpose
//                WT [K x N] for the backward data product
//   gradients    dZ [M x N] bf16 (loss gradient w.r.t. a layer's
//                pre-activation)
// Forward  Y = tanh(X W^T + b)            gemm_nn, EPI_TANH
// Output   dZ = s (X W^T + b - T)          gemm_nn, EPI_LOSS (and the loss)
// Backward dZprev = (dZ W) * (1 - Yprev^2) gemm_nn on WT, EPI_DTANH
// Weights  G = dZ^T X                      gemm_tn, split over the samples
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>

#include "mlp.h"

namespace bcg {
namespace {

constexpr int BM = 128, BN = 128, BK = 64, NT = 256;
constexpr int PA = BK + 8;     // shared-memory pitch of the NN tiles (144 bytes: conflict-free ldmatrix rows)
constexpr int PT = BN + 8;     // pitch of the TN tiles (272 bytes)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(dst)), "l"(src));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(smem_u32(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3) : "r"(smem_u32(p)));
}
__device__ __forceinline__ void mma_bf16(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
               "{%0,%1,%2,%3};\n"
               : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ---------------------------------------------------------------------------
// C[M x N] = A[M x K] B[N x K]^T with a fused epilogue.  CTA tile 128 x 128,
// 8 warps as 2 (rows) x 4 (columns), warp tile 64 x 32 = 4 x 4 mma tiles;
// K in chunks of 64, two shared-memory stages filled by cp.async.
struct NNArgs {
  const __nv_bfloat16* a;    // [M x K]
  const __nv_bfloat16* b;    // [N x K]
  const float* bias;         // [N] or null
  const __nv_bfloat16* yprev;// EPI_DTANH: [M x N] activation whose derivative scales the product
  const float* target;       // EPI_LOSS: [M x nout] (null: inference, write the output only)
  __nv_bfloat16* out_bf;     // EPI_TANH / EPI_DTANH / EPI_LOSS (dZ): [M x N]
  float* out_f32;            // EPI_LOSS: [M x nout] output values, may be null
  float* loss_part;          // EPI_LOSS with target: one partial sum of squares per CTA
  int m, n, k, nout, m_valid;// rows >= m_valid are padding: zero gradient, no loss
  float gscale;
};

template <int EPI>
__global__ void __launch_bounds__(NT) k_gemm_nn(NNArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16* sa = reinterpret_cast<__nv_bfloat16*>(smem_raw);   // [2][BM][PA]
  __nv_bfloat16* sb = sa + 2 * BM * PA;                               // [2][BN][PA]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 1, wn = warp >> 1;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int nk = p.k / BK;

  auto load = [&](int stage, int kc) {
    const int k0 = kc * BK;
#pragma unroll
    for (int r = 0; r < 4; ++r) {  // 128 rows x 8 chunks of 16 bytes, 4 per thread, for A and for B
      const int c = tid + r * NT, row = c >> 3, col = (c & 7) * 8;
      cp_async16(sa + (stage * BM + row) * PA + col, p.a + (size_t)(m0 + row) * p.k + k0 + col);
      cp_async16(sb + (stage * BN + row) * PA + col, p.b + (size_t)(n0 + row) * p.k + k0 + col);
    }
    cp_commit();
  };

  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

  load(0, 0);
  for (int kc = 0; kc < nk; ++kc) {
    if (kc + 1 < nk) {
      load((kc + 1) & 1, kc + 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    const __nv_bfloat16* ta = sa + (kc & 1) * BM * PA;
    const __nv_bfloat16* tb = sb + (kc & 1) * BN * PA;
#pragma unroll
    for (int ks = 0; ks < BK; ks += 16) {
      uint32_t af[4][4], bf[4][2];
#pragma unroll
      for (int mt = 0; mt < 4; ++mt) {
        const int row = wm * 64 + mt * 16 + (lane & 15), col = ks + (lane >> 4) * 8;
        ldsm_x4(af[mt][0], af[mt][1], af[mt][2], af[mt][3], ta + row * PA + col);
      }
#pragma unroll
      for (int np = 0; np < 2; ++np) {
        const int row = wn * 32 + np * 16 + (lane & 7) + ((lane >> 4) << 3), col = ks + ((lane >> 3) & 1) * 8;
        ldsm_x4(bf[2 * np][0], bf[2 * np][1], bf[2 * np + 1][0], bf[2 * np + 1][1], tb + row * PA + col);
      }
#pragma unroll
      for (int mt = 0; mt < 4; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], af[mt], bf[nt][0], bf[nt][1]);
    }
    __syncthreads();  // the stage just read is refilled by the next iteration's load
  }

  // epilogue: thread holds rows g, g+8 and columns 2q, 2q+1 of each 16 x 8 tile
  const int g = lane >> 2, q = lane & 3;
  float lsum = 0.f;
#pragma unroll
  for (int mt = 0; mt < 4; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = m0 + wm * 64 + mt * 16 + g + h * 8;
        const int col = n0 + wn * 32 + nt * 8 + 2 * q;
        float v0 = acc[mt][nt][2 * h], v1 = acc[mt][nt][2 * h + 1];
        if (p.bias) { v0 += p.bias[col]; v1 += p.bias[col + 1]; }
        const size_t o = (size_t)row * p.n + col;
        if (EPI == MLP_EPI_TANH) {
          *reinterpret_cast<__nv_bfloat162*>(p.out_bf + o) = __floats2bfloat162_rn(tanhf(v0), tanhf(v1));
        } else if (EPI == MLP_EPI_DTANH) {
          const __nv_bfloat162 y = *reinterpret_cast<const __nv_bfloat162*>(p.yprev + o);
          const float y0 = __low2float(y), y1 = __high2float(y);
          *reinterpret_cast<__nv_bfloat162*>(p.out_bf + o) =
              __floats2bfloat162_rn(v0 * (1.f - y0 * y0), v1 * (1.f - y1 * y1));
        } else {  // MLP_EPI_LOSS
          float d0 = 0.f, d1 = 0.f;
          const bool live = row < p.m_valid;
          if (col < p.nout) {
            if (p.out_f32) p.out_f32[(size_t)row * p.nout + col] = v0;
            if (p.target && live) d0 = v0 - p.target[(size_t)row * p.nout + col];
          }
          if (col + 1 < p.nout) {
            if (p.out_f32) p.out_f32[(size_t)row * p.nout + col + 1] = v1;
            if (p.target && live) d1 = v1 - p.target[(size_t)row * p.nout + col + 1];
          }
          lsum += d0 * d0 + d1 * d1;
          if (p.out_bf)
            *reinterpret_cast<__nv_bfloat162*>(p.out_bf + o) = __floats2bfloat162_rn(p.gscale * d0, p.gscale * d1);
        }
      }
  if (EPI == MLP_EPI_LOSS && p.loss_part) {
    __shared__ float red[NT / 32];
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, s);
    if (lane == 0) red[warp] = lsum;
    __syncthreads();
    if (tid == 0) {
      float t = 0.f;
      for (int w = 0; w < NT / 32; ++w) t += red[w];
      p.loss_part[blockIdx.y * gridDim.x + blockIdx.x] = t;
    }
  }
}

// ---------------------------------------------------------------------------
// P[z][N1 x N2] = sum over rows m of chunk z of A[m][n1] B[m][n2]
// (A = dZ [M x N1], B = X [M x N2]).  CTA tile 128 x 128; the rows of the
// chunk in steps of 64, two stages; both operands are read transposed from
// their row-major tiles by ldmatrix.trans.
struct TNArgs {
  const __nv_bfloat16* a;
  const __nv_bfloat16* b;
  float* part;  // [nsplit][N1][N2]
  int m, n1, n2, rows_per_split;
};

__global__ void __launch_bounds__(NT) k_gemm_tn(TNArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16* sa = reinterpret_cast<__nv_bfloat16*>(smem_raw);   // [2][BK][PT]
  __nv_bfloat16* sb = sa + 2 * BK * PT;                               // [2][BK][PT]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp & 1, wn = warp >> 1;
  const int i0 = blockIdx.y * BM, j0 = blockIdx.x * BN;
  const int r0 = blockIdx.z * p.rows_per_split;
  const int nk = p.rows_per_split / BK;

  auto load = [&](int stage, int kc) {
    const int rb = r0 + kc * BK;
#pragma unroll
    for (int r = 0; r < 4; ++r) {  // 64 rows x 16 chunks of 16 bytes
      const int c = tid + r * NT, row = c >> 4, col = (c & 15) * 8;
      cp_async16(sa + (stage * BK + row) * PT + col, p.a + (size_t)(rb + row) * p.n1 + i0 + col);
      cp_async16(sb + (stage * BK + row) * PT + col, p.b + (size_t)(rb + row) * p.n2 + j0 + col);
    }
    cp_commit();
  };

  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

  load(0, 0);
  for (int kc = 0; kc < nk; ++kc) {
    if (kc + 1 < nk) {
      load((kc + 1) & 1, kc + 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    const __nv_bfloat16* ta = sa + (kc & 1) * BK * PT;
    const __nv_bfloat16* tb = sb + (kc & 1) * BK * PT;
#pragma unroll
    for (int ks = 0; ks < BK; ks += 16) {
      uint32_t af[4][4], bf[4][2];
#pragma unroll
      for (int mt = 0; mt < 4; ++mt) {
        const int row = ks + (lane & 7) + ((lane >> 4) << 3);
        const int col = wm * 64 + mt * 16 + ((lane >> 3) & 1) * 8;
        ldsm_x4_t(af[mt][0], af[mt][1], af[mt][2], af[mt][3], ta + row * PT + col);
      }
#pragma unroll
      for (int np = 0; np < 2; ++np) {
        const int row = ks + (lane & 7) + (((lane >> 3) & 1) << 3);
        const int col = wn * 32 + np * 16 + (lane >> 4) * 8;
        ldsm_x4_t(bf[2 * np][0], bf[2 * np][1], bf[2 * np + 1][0], bf[2 * np + 1][1], tb + row * PT + col);
      }
#pragma unroll
      for (int mt = 0; mt < 4; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], af[mt], bf[nt][0], bf[nt][1]);
    }
    __syncthreads();
  }
  const int g = lane >> 2, q = lane & 3;
  float* out = p.part + (size_t)blockIdx.z * p.n1 * p.n2;
#pragma unroll
  for (int mt = 0; mt < 4; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = i0 + wm * 64 + mt * 16 + g + h * 8;
        const int col = j0 + wn * 32 + nt * 8 + 2 * q;
        *reinterpret_cast<float2*>(out + (size_t)row * p.n2 + col) =
            make_float2(acc[mt][nt][2 * h], acc[mt][nt][2 * h + 1]);
      }
}

// column sums of dZ [M x N] over row chunks: part[z][n]
__global__ void k_colsum(const __nv_bfloat16* __restrict__ dz, int m, int n, int rows_per_split,
                         float* __restrict__ part) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= n) return;
  const int r0 = blockIdx.y * rows_per_split;
  const int r1 = min(m, r0 + rows_per_split);
  float s = 0.f;
  for (int r = r0; r < r1; ++r) s += __bfloat162float(dz[(size_t)r * n + col]);
  part[(size_t)blockIdx.y * n + col] = s;
}

// gradient = fixed-order sum of the partials, then Adam on the FP32 master
// copy; writes the BF16 weights and their transpose.  Elements
// [0, n1 n2) are the weights (row o, column i), [n1 n2, n1 n2 + n1) the bias.
__global__ void k_adam(const float* __restrict__ wpart, int nsplit, const float* __restrict__ bpart, int bsplit,
                       int n1, int n2, float* __restrict__ w, float* __restrict__ mw, float* __restrict__ vw,
                       float* __restrict__ b, float* __restrict__ mb, float* __restrict__ vb,
                       __nv_bfloat16* __restrict__ wbf, __nv_bfloat16* __restrict__ wtbf, float lr, float beta1,
                       float beta2, float eps, float* __restrict__ grad_out) {
  const size_t nw = (size_t)n1 * n2;
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nw + n1) return;
  float gsum = 0.f;
  if (e < nw) {
    for (int z = 0; z < nsplit; ++z) gsum += wpart[(size_t)z * nw + e];
  } else {
    const int o = (int)(e - nw);
    for (int z = 0; z < bsplit; ++z) gsum += bpart[(size_t)z * n1 + o];
  }
  if (grad_out) grad_out[e] = gsum;
  if (lr == 0.f) return;  // gradient only
  float* pw = e < nw ? w + e : b + (e - nw);
  float* pm = e < nw ? mw + e : mb + (e - nw);
  float* pv = e < nw ? vw + e : vb + (e - nw);
  const float m1 = beta1 * *pm + (1.f - beta1) * gsum;
  const float v1 = beta2 * *pv + (1.f - beta2) * gsum * gsum;
  *pm = m1;
  *pv = v1;
  const float nwv = *pw - lr * m1 / (sqrtf(v1) + eps);  // lr carries the bias corrections
  *pw = nwv;
  if (e < nw) {
    const int o = (int)(e / n2), i = (int)(e % n2);
    const __nv_bfloat16 h = __float2bfloat16_rn(nwv);
    wbf[e] = h;
    wtbf[(size_t)i * n1 + o] = h;
  }
}

// FP32 master -> BF16 weights and transpose (after initialisation)
__global__ void k_cast_w(const float* __restrict__ w, int n1, int n2, __nv_bfloat16* __restrict__ wbf,
                         __nv_bfloat16* __restrict__ wtbf) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (size_t)n1 * n2) return;
  const int o = (int)(e / n2), i = (int)(e % n2);
  const __nv_bfloat16 h = __float2bfloat16_rn(w[e]);
  wbf[e] = h;
  wtbf[(size_t)i * n1 + o] = h;
}

// ---------------------------------------------------------------------------
// input features of one sample (cell c of parameter set s), MLP_NFEAT = 128:
//   0: 1;  1: rho;  2: a;  3: b  (rho = normalised log radius, a and b the
//   normalised Reynolds and Mach numbers, all in [0, 1])
//   4..51:   sin(k theta), cos(k theta), k = 1..24
//   52..99:  sin(pi k rho), cos(pi k rho), k = 1..24
//   100..123: sin(pi k a), cos(pi k a), sin(pi k b), cos(pi k b), k = 1..6
//   124: a b;  125: rho a;  126: rho b;  127: 0
__device__ void features(float theta, float rho, float a, float b, __nv_bfloat16* f) {
  const float pi = 3.14159265358979f;
  f[0] = __float2bfloat16_rn(1.f);
  f[1] = __float2bfloat16_rn(rho);
  f[2] = __float2bfloat16_rn(a);
  f[3] = __float2bfloat16_rn(b);
  for (int k = 1; k <= 24; ++k) {
    float s, c;
    sincosf(k * theta, &s, &c);
    f[4 + 2 * (k - 1)] = __float2bfloat16_rn(s);
    f[5 + 2 * (k - 1)] = __float2bfloat16_rn(c);
    sincosf(pi * k * rho, &s, &c);
    f[52 + 2 * (k - 1)] = __float2bfloat16_rn(s);
    f[53 + 2 * (k - 1)] = __float2bfloat16_rn(c);
  }
  for (int k = 1; k <= 6; ++k) {
    float s, c;
    sincosf(pi * k * a, &s, &c);
    f[100 + 4 * (k - 1)] = __float2bfloat16_rn(s);
    f[101 + 4 * (k - 1)] = __float2bfloat16_rn(c);
    sincosf(pi * k * b, &s, &c);
    f[102 + 4 * (k - 1)] = __float2bfloat16_rn(s);
    f[103 + 4 * (k - 1)] = __float2bfloat16_rn(c);
  }
  f[124] = __float2bfloat16_rn(a * b);
  f[125] = __float2bfloat16_rn(rho * a);
  f[126] = __float2bfloat16_rn(rho * b);
  f[127] = __float2bfloat16_rn(0.f);
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // SplitMix64 finaliser (Steele, Lea, Flood 2014)
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// one row per sample.  Training (seed >= 0): sample = hash(seed, row) mod
// (nset ncell); inference (seed < 0): row r is cell r of set `set`.
__global__ void k_features(const float* __restrict__ theta, const float* __restrict__ rho, int ncell,
                           const float* __restrict__ params, int nset, const float* __restrict__ targets, int nout,
                           long long seed, int set, int m, int m_valid, __nv_bfloat16* __restrict__ x,
                           float* __restrict__ t) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  __nv_bfloat16* f = x + (size_t)r * MLP_NFEAT;
  if (r >= m_valid) {
    for (int k = 0; k < MLP_NFEAT; ++k) f[k] = __float2bfloat16_rn(0.f);
    if (t)
      for (int v = 0; v < nout; ++v) t[(size_t)r * nout + v] = 0.f;
    return;
  }
  int s, c;
  if (seed >= 0) {
    const uint64_t h = mix64((uint64_t)seed * 0x100000001b3ull + (uint64_t)r);
    const uint64_t idx = h % ((uint64_t)nset * ncell);
    s = (int)(idx / ncell);
    c = (int)(idx % ncell);
  } else {
    s = set;
    c = r;
  }
  features(theta[c], rho[c], params[2 * s], params[2 * s + 1], f);
  if (t && targets)
    for (int v = 0; v < nout; ++v) t[(size_t)r * nout + v] = targets[((size_t)s * ncell + c) * nout + v];
}

__global__ void k_sum(const float* __restrict__ x, int n, float* __restrict__ out) {
  __shared__ float red[32];
  float s = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += x[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    *out = t;
  }
}

}  // namespace

constexpr size_t kSmemNN = (size_t)2 * (BM + BN) * PA * 2;
constexpr size_t kSmemTN = (size_t)2 * 2 * BK * PT * 2;

cudaError_t mlp_gemm_nn(int epi, const void* a, const void* b, const float* bias, const void* yprev,
                        const float* target, void* out_bf, float* out_f32, float* loss_part, int m, int n, int k,
                        int nout, int m_valid, float gscale, cudaStream_t st) {
  static const cudaError_t attr = [] {  // once per process (thread-safe static initialisation)
    cudaError_t e = cudaFuncSetAttribute(k_gemm_nn<MLP_EPI_TANH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kSmemNN);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_gemm_nn<MLP_EPI_DTANH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemNN);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_gemm_nn<MLP_EPI_LOSS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemNN);
    return e;
  }();
  if (attr != cudaSuccess) return attr;
  NNArgs p{};
  p.a = (const __nv_bfloat16*)a; p.b = (const __nv_bfloat16*)b; p.bias = bias;
  p.yprev = (const __nv_bfloat16*)yprev; p.target = target; p.out_bf = (__nv_bfloat16*)out_bf;
  p.out_f32 = out_f32; p.loss_part = loss_part; p.m = m; p.n = n; p.k = k; p.nout = nout; p.m_valid = m_valid;
  p.gscale = gscale;
  const dim3 grid(n / BN, m / BM);
  switch (epi) {
    case MLP_EPI_TANH: k_gemm_nn<MLP_EPI_TANH><<<grid, NT, kSmemNN, st>>>(p); break;
    case MLP_EPI_DTANH: k_gemm_nn<MLP_EPI_DTANH><<<grid, NT, kSmemNN, st>>>(p); break;
    default: k_gemm_nn<MLP_EPI_LOSS><<<grid, NT, kSmemNN, st>>>(p); break;
  }
  return cudaGetLastError();
}

cudaError_t mlp_gemm_tn(const void* a, const void* b, float* part, int m, int n1, int n2, int nsplit,
                        cudaStream_t st) {
  static const cudaError_t attr =
      cudaFuncSetAttribute(k_gemm_tn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTN);
  if (attr != cudaSuccess) return attr;
  TNArgs p{(const __nv_bfloat16*)a, (const __nv_bfloat16*)b, part, m, n1, n2, m / nsplit};
  k_gemm_tn<<<dim3(n2 / BN, n1 / BM, nsplit), NT, kSmemTN, st>>>(p);
  return cudaGetLastError();
}

cudaError_t mlp_colsum(const void* dz, int m, int n, int nsplit, float* part, cudaStream_t st) {
  k_colsum<<<dim3((n + 127) / 128, nsplit), 128, 0, st>>>((const __nv_bfloat16*)dz, m, n, (m + nsplit - 1) / nsplit,
                                                          part);
  return cudaGetLastError();
}

cudaError_t mlp_adam(const float* wpart, int nsplit, const float* bpart, int bsplit, int n1, int n2, float* w,
                     float* mw, float* vw, float* b, float* mb, float* vb, void* wbf, void* wtbf, float lr,
                     float beta1, float beta2, float eps, float* grad_out, cudaStream_t st) {
  const size_t ne = (size_t)n1 * n2 + n1;
  k_adam<<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(wpart, nsplit, bpart, bsplit, n1, n2, w, mw, vw, b, mb, vb,
                                                       (__nv_bfloat16*)wbf, (__nv_bfloat16*)wtbf, lr, beta1, beta2,
                                                       eps, grad_out);
  return cudaGetLastError();
}

cudaError_t mlp_cast_weights(const float* w, int n1, int n2, void* wbf, void* wtbf, cudaStream_t st) {
  const size_t ne = (size_t)n1 * n2;
  k_cast_w<<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(w, n1, n2, (__nv_bfloat16*)wbf, (__nv_bfloat16*)wtbf);
  return cudaGetLastError();
}

cudaError_t mlp_features(const float* theta, const float* rho, int ncell, const float* params, int nset,
                         const float* targets, int nout, long long seed, int set, int m, int m_valid, void* x,
                         float* t, cudaStream_t st) {
  k_features<<<(m + 127) / 128, 128, 0, st>>>(theta, rho, ncell, params, nset, targets, nout, seed, set, m, m_valid,
                                              (__nv_bfloat16*)x, t);
  return cudaGetLastError();
}

cudaError_t mlp_sum(const float* x, int n, float* out, cudaStream_t st) {
  k_sum<<<1, 1024, 0, st>>>(x, n, out);
  return cudaGetLastError();
}

}  // namespace bcg

// ---------------------------------------------------------------------------
// C ABI: device arrays only, queued on the library stream, no synchronisation.
#include <initializer_list>
#include "runtime.h"

namespace {
bool dev_ok() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) { cudaGetLastError(); return false; }
  return true;
}
bool all_device(std::initializer_list<const void*> ptrs) {
  for (const void* p : ptrs)
    if (p && !bcg::is_device_ptr(p)) return false;
  return true;
}
}  // namespace

extern "C" {

int bcg_mlp_gemm_nn(int epi, const void* a, const void* b, const float* bias, const void* yprev, const float* target,
                    void* out_bf, float* out_f32, float* loss_part, int m, int n, int k, int nout, int m_valid,
                    float gscale) {
  using namespace bcg;
  if (!dev_ok()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (epi < MLP_EPI_TANH || epi > MLP_EPI_LOSS) return fail_arg("mlp_gemm_nn: unknown epilogue");
  if (m <= 0 || n <= 0 || k <= 0 || m % BM || n % BN || k % BK)
    return fail_arg("mlp_gemm_nn: need m, n multiples of 128 and k a multiple of 64");
  if (!a || !b) return fail_arg("mlp_gemm_nn: null operand");
  if (epi == MLP_EPI_DTANH && (!yprev || !out_bf)) return fail_arg("mlp_gemm_nn: DTANH needs yprev and out_bf");
  if (epi == MLP_EPI_TANH && !out_bf) return fail_arg("mlp_gemm_nn: TANH needs out_bf");
  if (epi == MLP_EPI_LOSS && (nout < 1 || nout > n || m_valid < 0 || m_valid > m))
    return fail_arg("mlp_gemm_nn: LOSS needs 1 <= nout <= n and 0 <= m_valid <= m");
  if (!all_device({a, b, bias, yprev, target, out_bf, out_f32, loss_part}))
    return fail_arg("mlp_gemm_nn: every array must be a device pointer");
  cudaError_t e = mlp_gemm_nn(epi, a, b, bias, yprev, target, out_bf, out_f32, loss_part, m, n, k, nout, m_valid,
                              gscale, current_stream());
  return e == cudaSuccess ? BCG_OK : fail_cuda("mlp_gemm_nn", e);
}

int bcg_mlp_gemm_tn(const void* dz, const void* x, float* part, int m, int n1, int n2, int nsplit) {
  using namespace bcg;
  if (!dev_ok()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (m <= 0 || nsplit <= 0 || m % (BK * nsplit) || n1 <= 0 || n2 <= 0 || n1 % BM || n2 % BN)
    return fail_arg("mlp_gemm_tn: need m a multiple of 64 nsplit and n1, n2 multiples of 128");
  if (!dz || !x || !part || !all_device({dz, x, part})) return fail_arg("mlp_gemm_tn: device arrays required");
  cudaError_t e = mlp_gemm_tn(dz, x, part, m, n1, n2, nsplit, current_stream());
  return e == cudaSuccess ? BCG_OK : fail_cuda("mlp_gemm_tn", e);
}

int bcg_mlp_colsum(const void* dz, int m, int n, int nsplit, float* part) {
  using namespace bcg;
  if (!dev_ok()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (m <= 0 || n <= 0 || nsplit <= 0 || nsplit > m) return fail_arg("mlp_colsum: bad extents");
  if (!dz || !part || !all_device({dz, part})) return fail_arg("mlp_colsum: device arrays required");
  cudaError_t e = mlp_colsum(dz, m, n, nsplit, part, current_stream());
  return e == cudaSuccess ? BCG_OK : fail_cuda("mlp_colsum", e);
}

int bcg_mlp_adam(const float* wpart, int nsplit, const float* bpart, int bsplit, int n1, int n2, float* w, float* mw,
                 float* vw, float* b, float* mb, float* vb, void* wbf, void* wtbf, float lr, float beta1, float beta2,
                 float eps, float* grad_out) {
  using namespace bcg;
  if (!dev_ok()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (n1 <= 0 || n2 <= 0 || nsplit <= 0 || bsplit <= 0 || !wpart || !bpart) return fail_arg("mlp_adam: bad extents");
  if (lr != 0.f && (!w || !mw || !vw || !b || !mb || !vb || !wbf || !wtbf))
    return fail_arg("mlp_adam: an update needs the weights, moments and BF16 copies");
  if (!all_device({wpart, bpart, w, mw, vw, b, mb, vb, wbf, wtbf, grad_out}))
    return fail_arg("mlp_adam: every array must be a device pointer");
  cudaError_t e = mlp_adam(wpart, nsplit, bpart, bsplit, n1, n2, w, mw, vw, b, mb, vb, wbf, wtbf, lr, beta1, beta2,
                           eps, grad_out, current_stream());
  return e == cudaSuccess ? BCG_OK : fail_cuda("mlp_adam", e);
}

int bcg_mlp_cast_weights(const float* w, int n1, int n2, void* wbf, void* wtbf) {
  using namespace bcg;
  if (!dev_ok()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (n1 <= 0 || n2 <= 0 || !w || !wbf || !wtbf || !all_device({w, wbf, wtbf}))
    return fail_arg("mlp_cast_weights: device arrays and positive extents required");
  cudaError_t e = mlp_cast_weights(w, n1, n2, wbf, wtbf, current_stream());
  return e == cudaSuccess ? BCG_OK : fail_cuda("mlp_cast_weights", e);
}

int bcg_mlp_features(const float* theta, const float* rho, int ncell, const float* params, int nset,
                     const float* targets, int nout, long long seed, int set, int m, int m_valid, void* x, float* t) {
  using namespace bcg;
  if (!dev_ok()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (ncell <= 0 || nset <= 0 || m <= 0 || m_valid < 0 || m_valid > m || nout < 1)
    return fail_arg("mlp_features: bad extents");
  if (seed < 0 && (set < 0 || set >= nset || m_valid > ncell))
    return fail_arg("mlp_features: inference needs 0 <= set < nset and m_valid <= ncell");
  if (!theta || !rho || !params || !x || !all_device({theta, rho, params, targets, x, t}))
    return fail_arg("mlp_features: device arrays required");
  cudaError_t e = mlp_features(theta, rho, ncell, params, nset, targets, nout, seed, set, m, m_valid, x, t,
                               current_stream());
  return e == cudaSuccess ? BCG_OK : fail_cuda("mlp_features", e);
}

int bcg_mlp_sum(const float* x, int n, float* out) {
  using namespace bcg;
  if (!dev_ok()) return fail_arg("no CUDA device"), BCG_ERR_NODEV;
  if (n <= 0 || !x || !out || !all_device({x, out})) return fail_arg("mlp_sum: device arrays required");
  cudaError_t e = mlp_sum(x, n, out, current_stream());
  return e == cudaSuccess ? BCG_OK : fail_cuda("mlp_sum", e);
}

}  // extern "C"
