// Colored Jacobian seeding and COO indexing (misc/ComputeJacobian.f90) and the
// residual norms (srcfv/norm.F90) on the device.
#include "assembly.h"
#include <cfloat>
#include <cmath>

namespace bcg {

// testvector (ComputeJacobian.f90:357-374) and testvector_partial (:1075-1092)
__global__ void k_testvector(double* __restrict__ wd, int m, int l, int k, int gh, int im, int jm, int istart,
                             int iend, int jstart, int jend, bool partial) {
  const int ni = im + 2 * gh, nj = jm + 2 * gh;
  const size_t n = (size_t)ni * nj * 5;
  const int step = 1 + 2 * gh;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(q % ni) + 1 - gh;
    const int j = (int)((q / ni) % nj) + 1 - gh;
    const int v = (int)(q / ((size_t)ni * nj));
    bool seed;
    if (!partial) seed = (v == m) && j >= k + 1 && j <= jm && (j - k - 1) % step == 0 && i >= l + 1 && i <= im &&
                         (i - l - 1) % step == 0;
    else seed = (v == m) && j >= jstart + k + 1 && j <= jend + 1 && (j - jstart - k - 1) % step == 0 &&
                i >= istart + l + 1 && i <= iend + 1 && (i - istart - l - 1) % step == 0;
    wd[q] = seed ? 1.0 : 0.0;
  }
}

long long jac_slot_base(int mode, int m, int l, int k, int gh, int im, int jm, int n) {
  const long long step = 1 + 2 * gh, c = (long long)im * jm * 5;
  long long b = (long long)k * c + (long long)l * c * step + (long long)m * c * step * step;
  if (mode == JAC_CHECK) b += (long long)n * c * 5 * step * step;
  return b;
}

// one thread per (i, j, e) slot of the seed
__global__ void k_computejacobian(JacArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int im = a.im, jm = a.jm, gh = a.gh;
  if (t >= im * jm * 5) return;
  const int i = 1 + t % im, j = 1 + (t / im) % jm, e = 1 + t / (im * jm);
  const int step = 1 + 2 * gh;
  const int ni = im + 2 * gh;
  const size_t np = (size_t)ni * (jm + 2 * gh);
  const double r = a.resd[(size_t)(i + gh - 1) + (size_t)(j + gh - 1) * ni + (size_t)(e - 1) * np];
  const double cd = a.coefdiag ? a.coefdiag[(i - 1) + (size_t)(j - 1) * im] : 0.0;
  const int m = a.m, l = a.l, k = a.k;
  const int row = e - 1 + (j - 1) * 5 + (i - 1) * jm * 5;
  const bool jn = (a.mode == JAC_RELAXED_WITHJN || a.mode == JAC_WITHJN || a.mode == JAC_CHECK);
  const int bad = jn ? 5 * im * jm - 2 : 5 * im * jm - 1;
  int valj, vali;
  if (a.mode == JAC_DZ) {
    if (k <= gh) valj = (j <= k + 1 + gh) ? k : (j - (k + 1) + gh) / step * step + k;
    else valj = (j <= k - gh) ? jm + 1 : (j - (k + 1) + gh) / step * step + k;
  } else {
    valj = (j <= k + 1 + gh) ? k : (j - gh - (k + 1) + 2 * gh) / step * step + k;
  }
  if (valj >= jm) { a.ia[t] = bad; a.ja[t] = 0; a.jac[t] = 0.0; return; }
  if (l <= gh) vali = (i <= l + 1 + gh) ? l : (i - (l + 1) + gh) / step * step + l;
  else if (i <= l - gh) vali = (a.mode == JAC_CHECK) ? l : (jn ? im - 1 - 2 * gh + l : im + 1);
  else vali = (i - (l + 1) + gh) / step * step + l;
  if (a.mode == JAC_CHECK) {
    // two-zone periodic variant with the |jac| < mini occupancy check
    const double old = a.jac[t];
    const bool free_slot = fabs(old) < a.mini;
    bool write = false, kill = false;
    if (a.n == 0) {
      if (vali >= im - 2 * gh) { vali = l; if (free_slot) write = true; else kill = true; }
      else if (free_slot) write = true;
    } else {
      if (vali <= 2 * gh) {
        vali = im - (im % step) + l;
        if (vali > im - 1) vali = vali - step;
        if (free_slot) write = true;
      } else { if (free_slot) write = true; else kill = true; }
    }
    a.ia[t] = row;
    if (write) {
      const int col = m + valj * 5 + vali * jm * 5;
      a.ja[t] = col;
      a.jac[t] = (row == col) ? cd - r : -r;
    } else if (kill) { a.ia[t] = bad; a.ja[t] = 0; a.jac[t] = 0.0; }
    return;
  }
  if (vali >= im) {
    if (jn && vali - im <= gh - 1) vali = l;
    else { a.ia[t] = bad; a.ja[t] = 0; a.jac[t] = 0.0; return; }
  }
  const int col = m + valj * 5 + vali * jm * 5;
  a.ia[t] = row;
  a.ja[t] = col;
  if (a.mode == JAC_DZ) a.jac[t] = r;
  else if ((a.mode == JAC_RELAXED || a.mode == JAC_RELAXED_WITHJN) && row == col) a.jac[t] = cd - r;
  else a.jac[t] = -r;
}

cudaError_t launch_computejacobian(const JacArgs& a, cudaStream_t st) {
  const int n = a.im * a.jm * 5, B = 256;
  k_computejacobian<<<(n + B - 1) / B, B, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_testvector(double* wd, int m, int l, int k, int gh, int im, int jm, int istart, int iend,
                              int jstart, int jend, bool partial, cudaStream_t st) {
  const size_t n = (size_t)(im + 2 * gh) * (jm + 2 * gh) * 5;
  const int B = 256;
  const unsigned nb = (unsigned)((n + B - 1) / B < 4096 ? (n + B - 1) / B : 4096);
  k_testvector<<<nb, B, 0, st>>>(wd, m, l, k, gh, im, jm, istart, iend, jstart, jend, partial);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// norms: per-block partials (sum x^2, sum x^10, max |x| with first index) of
// the 5 variables, then one block reduces them in a fixed order.
struct NormAcc { double s2[5], s10[5], mx[5]; long long ix[5]; };

__device__ inline void acc_merge(NormAcc& a, const NormAcc& b) {
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    a.s2[v] += b.s2[v];
    a.s10[v] += b.s10[v];
    if (b.mx[v] > a.mx[v] || (b.mx[v] == a.mx[v] && b.ix[v] < a.ix[v])) { a.mx[v] = b.mx[v]; a.ix[v] = b.ix[v]; }
  }
}

__device__ inline void warp_merge(NormAcc& a) {
  for (int o = 16; o > 0; o >>= 1) {
    NormAcc b;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      b.s2[v] = __shfl_down_sync(0xffffffffu, a.s2[v], o);
      b.s10[v] = __shfl_down_sync(0xffffffffu, a.s10[v], o);
      b.mx[v] = __shfl_down_sync(0xffffffffu, a.mx[v], o);
      b.ix[v] = __shfl_down_sync(0xffffffffu, a.ix[v], o);
    }
    acc_merge(a, b);
  }
}

constexpr int kNormThreads = 256;
constexpr int kPartialDoubles = 20;  // s2, s10, mx, ix(as double) x 5

__global__ void __launch_bounds__(kNormThreads) k_norm_partial(const double* __restrict__ rhs, int im, int jm, int gh,
                                                               double* __restrict__ part) {
  const int ni = im + 2 * gh;
  const size_t np = (size_t)ni * (jm + 2 * gh);
  const long long n = (long long)im * jm;
  NormAcc a;
#pragma unroll
  for (int v = 0; v < 5; ++v) { a.s2[v] = 0.0; a.s10[v] = 0.0; a.mx[v] = -1.0; a.ix[v] = LLONG_MAX; }
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % im), j = 1 + (int)(t / im);
    const size_t q = (size_t)(i + gh - 1) + (size_t)(j + gh - 1) * ni;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double x = __ldg(rhs + q + (size_t)v * np);
      const double x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;
      a.s2[v] += x2;
      a.s10[v] += x8 * x2;
      const double ax = fabs(x);
      if (ax > a.mx[v]) { a.mx[v] = ax; a.ix[v] = t; }
    }
  }
  warp_merge(a);
  __shared__ NormAcc sh[kNormThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    NormAcc b = sh[0];
    for (int k = 1; k < kNormThreads / 32; ++k) acc_merge(b, sh[k]);
    double* o = part + (size_t)blockIdx.x * kPartialDoubles;
    for (int v = 0; v < 5; ++v) { o[v] = b.s2[v]; o[5 + v] = b.s10[v]; o[10 + v] = b.mx[v]; o[15 + v] = (double)b.ix[v]; }
  }
}

__global__ void k_norm_final(const double* __restrict__ part, int nb, int kind, const double* __restrict__ rhs,
                             int im, int jm, int gh, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  NormAcc a;
  for (int v = 0; v < 5; ++v) { a.s2[v] = 0.0; a.s10[v] = 0.0; a.mx[v] = -1.0; a.ix[v] = LLONG_MAX; }
  for (int b = 0; b < nb; ++b) {
    const double* o = part + (size_t)b * kPartialDoubles;
    NormAcc c;
    for (int v = 0; v < 5; ++v) { c.s2[v] = o[v]; c.s10[v] = o[5 + v]; c.mx[v] = o[10 + v]; c.ix[v] = (long long)o[15 + v]; }
    acc_merge(a, c);
  }
  const int ni = im + 2 * gh;
  const size_t np = (size_t)ni * (jm + 2 * gh);
  const long long last = (long long)im * jm - 1;
  for (int v = 0; v < 5; ++v) {
    if (kind == NORM_L2) { out[v] = sqrt(a.s2[v]); out[5 + v] = out[v] / (double)(im * jm); }
    else if (kind == NORM_L2INF) { out[v] = sqrt(a.s2[v]); out[5 + v] = pow(a.s10[v], 0.1); }
    else {
      // compute_maxnorm keeps the signed value only when the maximum sits at
      // the last visited cell (norm.F90:98-104); zero if never updated
      if (a.mx[v] <= 0.0) { out[v] = 0.0; out[5 + v] = -1; out[10 + v] = -1; continue; }
      const long long t = a.ix[v];
      const int i = 1 + (int)(t % im), j = 1 + (int)(t / im);
      const double x = rhs[(size_t)(i + gh - 1) + (size_t)(j + gh - 1) * ni + (size_t)v * np];
      out[v] = (t == last) ? x : fabs(x);
      out[5 + v] = i;
      out[10 + v] = j;
    }
  }
}

int norm_partial_blocks(int im, int jm) {
  long long n = (long long)im * jm;
  long long nb = (n + kNormThreads * 8 - 1) / (kNormThreads * 8);
  if (nb < 1) nb = 1;
  if (nb > 304) nb = 304;
  return (int)nb;
}

cudaError_t launch_norm(int kind, const double* rhs, int im, int jm, int gh, double* out, double* partial, int npartial,
                        cudaStream_t st) {
  k_norm_partial<<<npartial, kNormThreads, 0, st>>>(rhs, im, jm, gh, partial);
  k_norm_final<<<1, 32, 0, st>>>(partial, npartial, kind, rhs, im, jm, gh, out);
  return cudaGetLastError();
}

}  // namespace bcg
