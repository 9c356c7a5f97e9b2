// Test infrastructure only: scalar types for the CPU oracle of the BROADCAST
// DNC5 residual path.  Nothing in the shipped library includes this file.
//
// Dual<N>  : forward-mode dual number with N tangent directions.  The branch
//            conventions follow the ones the reference's Tapenade 3.16
//            tangent code uses, so a Dual<N> run of the restated primal
//            reproduces srcfv/tangent/*_d.f90 up to rounding:
//              abs(x)   : derivative +dx when x >= 0, else -dx
//                         (tangent/flux_num_dnc5_d.f90:945-951)
//              sqrt(x)  : derivative 0 when x == 0
//                         (tangent/flux_num_dnc5_d.f90:367-371)
//              max(a,b) : takes b (value and derivative) when a < b, else a
//                         (tangent/flux_num_dnc5_d.f90:1054-1060, 1117-1123)
//              x**y     : derivative 0 when x <= 0 and y is 0 or non-integer
//                         (tangent/bc_wall_viscous_d.f90:118-122)
//              sign(a,b): constant first argument, derivative 0
// OpCount  : tallies the floating-point operations of one evaluation by kind
//            (each +, -, *, / and each intrinsic counts one); used for the
//            algorithmic flop figure of the roofline.
#pragma once
#include <cmath>
#include <cstdint>

namespace orc {

template <int N>
struct Dual {
  double v;
  double d[N];
  Dual() : v(0.0) { for (int k = 0; k < N; ++k) d[k] = 0.0; }
  Dual(double x) : v(x) { for (int k = 0; k < N; ++k) d[k] = 0.0; }
};

template <int N> inline double val(const Dual<N>& a) { return a.v; }
inline double val(double a) { return a; }

template <int N> inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v + b.v; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k]; return r;
}
template <int N> inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v - b.v; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k]; return r;
}
template <int N> inline Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r; r.v = -a.v; for (int k = 0; k < N; ++k) r.d[k] = -a.d[k]; return r;
}
template <int N> inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v * b.v; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k]; return r;
}
template <int N> inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r; r.v = a.v / b.v;
  for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
  return r;
}
// mixed forms with a passive double
template <int N> inline Dual<N> operator+(const Dual<N>& a, double b) { Dual<N> r = a; r.v = a.v + b; return r; }
template <int N> inline Dual<N> operator+(double a, const Dual<N>& b) { Dual<N> r = b; r.v = a + b.v; return r; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, double b) { Dual<N> r = a; r.v = a.v - b; return r; }
template <int N> inline Dual<N> operator-(double a, const Dual<N>& b) {
  Dual<N> r; r.v = a - b.v; for (int k = 0; k < N; ++k) r.d[k] = -b.d[k]; return r;
}
template <int N> inline Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r; r.v = a.v * b; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b; return r;
}
template <int N> inline Dual<N> operator*(double a, const Dual<N>& b) {
  Dual<N> r; r.v = a * b.v; for (int k = 0; k < N; ++k) r.d[k] = a * b.d[k]; return r;
}
template <int N> inline Dual<N> operator/(const Dual<N>& a, double b) {
  Dual<N> r; r.v = a.v / b; for (int k = 0; k < N; ++k) r.d[k] = a.d[k] / b; return r;
}
template <int N> inline Dual<N> operator/(double a, const Dual<N>& b) {
  Dual<N> r; r.v = a / b.v; for (int k = 0; k < N; ++k) r.d[k] = -r.v * b.d[k] / b.v; return r;
}
template <int N> inline bool operator<(const Dual<N>& a, const Dual<N>& b) { return a.v < b.v; }
template <int N> inline bool operator<(const Dual<N>& a, double b) { return a.v < b; }
template <int N> inline bool operator<(double a, const Dual<N>& b) { return a < b.v; }
template <int N> inline bool operator>=(const Dual<N>& a, double b) { return a.v >= b; }

template <int N> inline Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r; r.v = std::sqrt(a.v);
  for (int k = 0; k < N; ++k) r.d[k] = (a.v == 0.0) ? 0.0 : a.d[k] / (2.0 * r.v);
  return r;
}
template <int N> inline Dual<N> abs(const Dual<N>& a) {
  if (a.v >= 0.0) return a;
  return -a;
}
template <int N> inline Dual<N> tanh(const Dual<N>& a) {
  Dual<N> r; r.v = std::tanh(a.v);
  const double s = 1.0 - r.v * r.v;
  for (int k = 0; k < N; ++k) r.d[k] = s * a.d[k];
  return r;
}
template <int N> inline Dual<N> pow(const Dual<N>& a, double y) {
  Dual<N> r; r.v = std::pow(a.v, y);
  const bool zero = (a.v <= 0.0) && (y == 0.0 || y != (double)(long long)y);
  const double s = zero ? 0.0 : y * std::pow(a.v, y - 1.0);
  for (int k = 0; k < N; ++k) r.d[k] = s * a.d[k];
  return r;
}
// Fortran MAX with the Tapenade derivative choice: b when a < b, else a.
template <class T> inline T fmax_t(const T& a, const T& b) { return (a < b) ? b : a; }
inline double fabs_t(double a) { return std::fabs(a); }
template <int N> inline Dual<N> fabs_t(const Dual<N>& a) { return abs(a); }
inline double sqrt_t(double a) { return std::sqrt(a); }
template <int N> inline Dual<N> sqrt_t(const Dual<N>& a) { return sqrt(a); }
inline double tanh_t(double a) { return std::tanh(a); }
template <int N> inline Dual<N> tanh_t(const Dual<N>& a) { return tanh(a); }
inline double pow_t(double a, double y) { return std::pow(a, y); }
template <int N> inline Dual<N> pow_t(const Dual<N>& a, double y) { return pow(a, y); }
// Fortran SIGN(a, b) for a passive magnitude: |a| with the sign of b; +|a|
// for b = +0 (borders/bc_no_reflexion.F90:72-74).
inline double fsign(double a, double b) { return (b >= 0.0) ? std::fabs(a) : -std::fabs(a); }
template <int N> inline double fsign(double a, const Dual<N>& b) { return fsign(a, b.v); }

// ---------------------------------------------------------------------------
// OpCount: a double that tallies the operations of one evaluation by kind.
// Active (A) operands carry derivatives, passive (P) ones are constants; the
// kinds are what the flop count of the tangent needs (oracle_capi.cpp).
enum OpKind {
  OP_ADD_AA = 0, OP_ADD_AP, OP_MUL_AA, OP_MUL_AP, OP_DIV_AA, OP_DIV_AP, OP_DIV_PA,
  OP_SQRT, OP_TANH, OP_ABS, OP_MAX, OP_POW, OP_NKIND
};
struct OpCount {
  double v;
  static inline uint64_t* tally() { static thread_local uint64_t t[OP_NKIND] = {0}; return t; }
  static inline void reset() { for (int k = 0; k < OP_NKIND; ++k) tally()[k] = 0; }
  OpCount() : v(0.0) {}
  OpCount(double x) : v(x) {}
};
inline double val(const OpCount& a) { return a.v; }
#define ORC_OPC_BIN(op, kaa, kap, kpa)                                                                           \
  inline OpCount operator op(const OpCount& a, const OpCount& b) { ++OpCount::tally()[kaa]; return OpCount(a.v op b.v); } \
  inline OpCount operator op(const OpCount& a, double b) { ++OpCount::tally()[kap]; return OpCount(a.v op b); }           \
  inline OpCount operator op(double a, const OpCount& b) { ++OpCount::tally()[kpa]; return OpCount(a op b.v); }
ORC_OPC_BIN(+, OP_ADD_AA, OP_ADD_AP, OP_ADD_AP)
ORC_OPC_BIN(-, OP_ADD_AA, OP_ADD_AP, OP_ADD_AP)
ORC_OPC_BIN(*, OP_MUL_AA, OP_MUL_AP, OP_MUL_AP)
ORC_OPC_BIN(/, OP_DIV_AA, OP_DIV_AP, OP_DIV_PA)
#undef ORC_OPC_BIN
inline OpCount operator-(const OpCount& a) { return OpCount(-a.v); }
inline bool operator<(const OpCount& a, const OpCount& b) { return a.v < b.v; }
inline bool operator<(const OpCount& a, double b) { return a.v < b; }
inline bool operator<(double a, const OpCount& b) { return a < b.v; }
inline bool operator>=(const OpCount& a, double b) { return a.v >= b; }
inline OpCount fabs_t(const OpCount& a) { ++OpCount::tally()[OP_ABS]; return OpCount(std::fabs(a.v)); }
inline OpCount sqrt_t(const OpCount& a) { ++OpCount::tally()[OP_SQRT]; return OpCount(std::sqrt(a.v)); }
inline OpCount tanh_t(const OpCount& a) { ++OpCount::tally()[OP_TANH]; return OpCount(std::tanh(a.v)); }
inline OpCount pow_t(const OpCount& a, double y) { ++OpCount::tally()[OP_POW]; return OpCount(std::pow(a.v, y)); }
inline OpCount fmax_t(const OpCount& a, const OpCount& b) { ++OpCount::tally()[OP_MAX]; return (a.v < b.v) ? b : a; }
inline double fsign(double a, const OpCount& b) { return fsign(a, b.v); }

}  // namespace orc
