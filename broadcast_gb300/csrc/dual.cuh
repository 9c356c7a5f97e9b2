// Device scalar types for the DNC5 kernels.
//
// The residual kernels are written once over a scalar type S:
//   S = double   : primal residual,
//   S = DK<K>    : primal plus K tangent directions (fused residual + JVP).
// Derivative conventions match the reference's Tapenade 3.16 tangent code
// (srcfv/tangent/flux_num_dnc5_d.f90): abs takes +dx at x >= 0
// (:945-951), sqrt has zero derivative at 0 (:367-371), MAX takes its second
// argument only when the first is strictly smaller (:1054-1060), x**y has zero
// derivative for x <= 0 with a non-integer y (tangent/bc_wall_viscous_d.f90:118).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace bcg {

template <int K>
struct DK {
  double v;
  double d[K];
};

#define BCG_HD __device__ __forceinline__

// 1/x correctly rounded (round to nearest): the device intrinsic, which
// yields the same value as the IEEE division 1.0/x with a shorter sequence
BCG_HD double rcp_rn(double x) {
#ifdef __CUDA_ARCH__
  return __drcp_rn(x);
#else
  return 1.0 / x;
#endif
}

template <int K> BCG_HD DK<K> mkc(double x) { DK<K> r; r.v = x;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = 0.0; return r; }

template <int K> BCG_HD double val(const DK<K>& a) { return a.v; }
BCG_HD double val(double a) { return a; }

template <int K> BCG_HD DK<K> operator+(const DK<K>& a, const DK<K>& b) { DK<K> r; r.v = a.v + b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k]; return r; }
template <int K> BCG_HD DK<K> operator-(const DK<K>& a, const DK<K>& b) { DK<K> r; r.v = a.v - b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k]; return r; }
template <int K> BCG_HD DK<K> operator-(const DK<K>& a) { DK<K> r; r.v = -a.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = -a.d[k]; return r; }
template <int K> BCG_HD DK<K> operator*(const DK<K>& a, const DK<K>& b) { DK<K> r; r.v = a.v * b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = fma(a.d[k], b.v, a.v * b.d[k]); return r; }
// Divisions take one IEEE reciprocal, shared by the value and the tangents
// (the value a * (1/b) is within an ulp of a / b).
template <int K> BCG_HD DK<K> operator/(const DK<K>& a, const DK<K>& b) {
  DK<K> r; const double inv = rcp_rn(b.v); r.v = a.v * inv;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = fma(-r.v, b.d[k], a.d[k]) * inv; return r; }

template <int K> BCG_HD DK<K> operator+(const DK<K>& a, double b) { DK<K> r = a; r.v = a.v + b; return r; }
template <int K> BCG_HD DK<K> operator+(double a, const DK<K>& b) { DK<K> r = b; r.v = a + b.v; return r; }
template <int K> BCG_HD DK<K> operator-(const DK<K>& a, double b) { DK<K> r = a; r.v = a.v - b; return r; }
template <int K> BCG_HD DK<K> operator-(double a, const DK<K>& b) { DK<K> r; r.v = a - b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = -b.d[k]; return r; }
template <int K> BCG_HD DK<K> operator*(const DK<K>& a, double b) { DK<K> r; r.v = a.v * b;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b; return r; }
template <int K> BCG_HD DK<K> operator*(double a, const DK<K>& b) { DK<K> r; r.v = a * b.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a * b.d[k]; return r; }
template <int K> BCG_HD DK<K> operator/(const DK<K>& a, double b) { DK<K> r; const double inv = rcp_rn(b); r.v = a.v * inv;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * inv; return r; }
template <int K> BCG_HD DK<K> operator/(double a, const DK<K>& b) {
  DK<K> r; const double inv = rcp_rn(b.v); r.v = a * inv; const double s = -r.v * inv;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = s * b.d[k]; return r; }

template <int K> BCG_HD bool operator<(const DK<K>& a, const DK<K>& b) { return a.v < b.v; }
template <int K> BCG_HD bool operator<(const DK<K>& a, double b) { return a.v < b; }
template <int K> BCG_HD bool operator<(double a, const DK<K>& b) { return a < b.v; }

template <int K> BCG_HD DK<K> sqrt_t(const DK<K>& a) { DK<K> r; r.v = sqrt(a.v);
  const double s = (a.v == 0.0) ? 0.0 : 0.5 * rcp_rn(r.v);  // = 0.5/r.v exactly
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * s; return r; }
BCG_HD double sqrt_t(double a) { return sqrt(a); }
// sqrt through one reciprocal square root: x rsqrt(x), derivative 0.5 rsqrt(x)
// (within 2 ulp of the correctly rounded sqrt; for the magnitudes that feed
// no branch: spectral radius, sqrt(rho), the Sutherland term)
template <int K> BCG_HD DK<K> sqrt_r(const DK<K>& a) { DK<K> r;
  const double rs = (a.v == 0.0) ? 0.0 : rsqrt(a.v);
  r.v = a.v * rs;
  const double s = 0.5 * rs;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * s; return r; }
BCG_HD double sqrt_r(double a) { return (a == 0.0) ? 0.0 : a * rsqrt(a); }
template <int K> BCG_HD DK<K> fabs_t(const DK<K>& a) { return (a.v >= 0.0) ? a : -a; }
BCG_HD double fabs_t(double a) { return fabs(a); }
template <int K> BCG_HD DK<K> tanh_t(const DK<K>& a) { DK<K> r; r.v = tanh(a.v); const double s = 1.0 - r.v * r.v;
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = s * a.d[k]; return r; }
BCG_HD double tanh_t(double a) { return tanh(a); }
template <int K> BCG_HD DK<K> pow_t(const DK<K>& a, double y) { DK<K> r; r.v = pow(a.v, y);
  const bool z = (a.v <= 0.0) && (y == 0.0 || y != trunc(y));
  const double s = z ? 0.0 : y * pow(a.v, y - 1.0);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = s * a.d[k]; return r; }
BCG_HD double pow_t(double a, double y) { return pow(a, y); }
template <class S> BCG_HD S fmax_t(const S& a, const S& b) { return (a < b) ? b : a; }

// Operations whose value is rounded as the separate IEEE operation, never
// contracted into a fused multiply-add, and a correctly rounded division.
// The pressure and the pressure sensor are formed with them in the
// reference's order: next to an extrapolated boundary the sensor's two
// ratios can agree to ~1e-7, so MAX(ks1, ks2) and with it the tangent's
// branch follow the last bits of the pressure (phys/Primitives.F,
// rhs/ducrosfordnc_i.F).
BCG_HD double mul_rn(double a, double b) { return __dmul_rn(a, b); }
BCG_HD double add_rn(double a, double b) { return __dadd_rn(a, b); }
BCG_HD double sub_rn(double a, double b) { return __dsub_rn(a, b); }
BCG_HD double div_rn(double a, double b) { return __ddiv_rn(a, b); }
template <int K> BCG_HD DK<K> mul_rn(const DK<K>& a, const DK<K>& b) { DK<K> r; r.v = __dmul_rn(a.v, b.v);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = fma(a.d[k], b.v, a.v * b.d[k]); return r; }
template <int K> BCG_HD DK<K> mul_rn(double a, const DK<K>& b) { DK<K> r; r.v = __dmul_rn(a, b.v);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a * b.d[k]; return r; }
template <int K> BCG_HD DK<K> add_rn(const DK<K>& a, const DK<K>& b) { DK<K> r; r.v = __dadd_rn(a.v, b.v);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k]; return r; }
template <int K> BCG_HD DK<K> sub_rn(const DK<K>& a, const DK<K>& b) { DK<K> r; r.v = __dsub_rn(a.v, b.v);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k]; return r; }
template <int K> BCG_HD DK<K> div_rn(const DK<K>& a, const DK<K>& b) {
  DK<K> r; r.v = __ddiv_rn(a.v, b.v); const double inv = rcp_rn(b.v);
#pragma unroll
  for (int k = 0; k < K; ++k) r.d[k] = fma(-r.v, b.d[k], a.d[k]) * inv; return r; }
BCG_HD double fsign(double a, double b) { return (b >= 0.0) ? fabs(a) : -fabs(a); }
template <int K> BCG_HD double fsign(double a, const DK<K>& b) { return fsign(a, b.v); }

// number of tangent directions carried by a scalar type
template <class S> struct NDir { static constexpr int value = 0; };
template <int K> struct NDir<DK<K>> { static constexpr int value = K; };

// constant of scalar type S
template <class S> BCG_HD S cst(double x);
template <> BCG_HD double cst<double>(double x) { return x; }
template <class S> struct CstHelper;
template <int K> BCG_HD DK<K> cstk(double x) { return mkc<K>(x); }

// Loads / stores of a scalar from K+1 planes of stride `plane` doubles:
// plane 0 holds the value, plane 1+k the k-th tangent.
template <class S> struct Planes;
template <> struct Planes<double> {
  BCG_HD static double ld(const double* __restrict__ p, size_t /*plane*/, size_t q) { return __ldg(p + q); }
  BCG_HD static void st(double* __restrict__ p, size_t /*plane*/, size_t q, double x) { p[q] = x; }
  BCG_HD static double zero() { return 0.0; }
  BCG_HD static double c(double x) { return x; }
};
template <int K> struct Planes<DK<K>> {
  BCG_HD static DK<K> ld(const double* __restrict__ p, size_t plane, size_t q) {
    DK<K> r; r.v = __ldg(p + q);
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = __ldg(p + (size_t)(k + 1) * plane + q);
    return r;
  }
  BCG_HD static void st(double* __restrict__ p, size_t plane, size_t q, const DK<K>& x) {
    p[q] = x.v;
#pragma unroll
    for (int k = 0; k < K; ++k) p[(size_t)(k + 1) * plane + q] = x.d[k];
  }
  BCG_HD static DK<K> zero() { return mkc<K>(0.0); }
  BCG_HD static DK<K> c(double x) { return mkc<K>(x); }
};

}  // namespace bcg
