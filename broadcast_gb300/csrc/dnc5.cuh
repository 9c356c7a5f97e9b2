// DNC5 residual building blocks (device side), written over a scalar type S
// (double, or DK<K> for the fused residual + K-direction JVP).
//
// Reference: srcfv/prepro/flux_num_dnc5.f90 (flattened form of
// srcfv/rhs/flux_num_dnc5.F90 and its rhs/ and phys/ fragments).
//
// Data layout (the reference's f2py layout, kept for zero-copy drop-in):
//   cell arrays  w, residu, vol, volf: Fortran order (1-gh:im+gh, 1-gh:jm+gh[, v])
//   face arrays  nx, ny             : (1-gh:im+gh+1, 1-gh:jm+gh+1, 2)
// The kernels work in three passes over HBM-resident scratch:
//   pass 1  cell primitives (u, v, w, T, p, mu, Euler fluxes f2..f5, g2..g5)
//           on every padded cell, once per cell;
//   pass 2  the sensor's cell quantities (pressure ratios, Ducros ratio from
//           the u and v gradients), once per cell of the interior and its
//           one-cell ghost ring;
//   pass 3  every face flux once (i- and j-faces of node (i,j)), then the
//           balance differences them into the residual.
#pragma once
#include "dual.cuh"

namespace bcg {

struct Phys {
  double cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4;
};

// scalar coefficients derived once on the host (flux_num_dnc5.f90:69-122, 938-950)
//
// The DNC schemes of order 3, 5, 7 and 9 (srcfv/rhs/flux_num_dnc{3,5,7,9}.F90)
// share every pass; they differ in R = (order+1)/2, the number of point pairs
// of their stencils, which the face kernels take as a template argument:
//   bb[0..R-2]   cell-gradient weights      (rhs/gradop_{3,5,7,9}p{i,j}.F)
//   cc[0..R-1]   centred face-flux weights  (rhs/euler_o{4,6,8,10}_{i,j}.F)
//   dd[0..R-1]   predictor weights          (rhs/predictor_{5,7,9,11}p_{i,j}.F)
//   cw[r][0..nw-1]  off-centred j-flux weights of wall row j = r + 2 over the
//                first nw cell rows (rhs/nearbndfluxes*demi_*.F with
//                rhs/coefnearbnd_{7,9,11}p.F; DNC3 averages rows 1 and 2)
// The named DNC5 fields below are kept for the DNC5-only kernels (adjoint).
struct Coef {
  double cpprandtl, cvm1, ccross, betas, gam1, c2fac;  // c2fac = gam*rgaz
  double b1, b2, c1, c2, c3, d1, d2, d3;
  double c5[5], c3w[5];
  double ct0, ct1, k2, k4, s_suth;
  int wall;  // 1: adiabatic wall at j = 1 (flux_num_dnc5_2d); 0: centred rows everywhere (flux_num_dnc5_nowall_2d)
  int order, nw;
  double bb[4], cc[5], dd[5], cw[4][11];
};

// number of point pairs of the DNC scheme of the given order (0 if none)
inline int dnc_pairs(int order) {
  return (order == 3 || order == 5 || order == 7 || order == 9) ? (order + 1) / 2 : 0;
}

// stencil weights of the DNC scheme of the given order, each formed with the
// floating-point operations the reference uses
inline void set_stencils(Coef& c, int order) {
  c.order = order;
  for (auto& x : c.bb) x = 0.0;
  for (auto& x : c.cc) x = 0.0;
  for (auto& x : c.dd) x = 0.0;
  for (auto& r : c.cw) for (auto& x : r) x = 0.0;
  double denom;
  if (order == 3) {  // flux_num_dnc3.F90:104-123, 172-173
    denom = 1.0 / 12.0;
    c.bb[0] = 0.5;
    c.cc[0] = 7.0 * denom; c.cc[1] = -denom;
    c.dd[0] = 3.0 * denom; c.dd[1] = denom;
    c.nw = 2;
    c.cw[0][0] = 0.5; c.cw[0][1] = 0.5;
  } else if (order == 7) {  // flux_num_dnc7.F90:92-128, rhs/coefnearbnd_9p.F (denom 1/840)
    denom = 1.0 / 60.0;
    c.bb[0] = 45.0 * denom; c.bb[1] = -9.0 * denom; c.bb[2] = denom;
    denom = 1.0 / 840.0;
    const double cc[4] = {533.0, -139.0, 29.0, -3.0};
    for (int n = 0; n < 4; ++n) c.cc[n] = cc[n] * denom;
    denom = 1.0 / 280.0;
    const double dd[4] = {35.0, 21.0, 7.0, 1.0};
    for (int n = 0; n < 4; ++n) c.dd[n] = dd[n] * denom;
    denom = 1.0 / 840.0;
    c.nw = 9;
    const double w3[9] = {92.0, 1547.0, -1861.0, 2171.0, -1917.0, 1191.0, -489.0, 119.0, -13.0};
    const double w5[9] = {-13.0, 209.0, 1079.0, -769.0, 533.0, -279.0, 99.0, -21.0, 2.0};
    const double w7[9] = {2.0, -31.0, 281.0, 911.0, -517.0, 281.0, -111.0, 27.0, -3.0};
    for (int n = 0; n < 9; ++n) { c.cw[0][n] = w3[n] * denom; c.cw[1][n] = w5[n] * denom; c.cw[2][n] = w7[n] * denom; }
  } else if (order == 9) {  // flux_num_dnc9.F90:100-128, rhs/coefnearbnd_11p.F
    denom = 1.0 / 840.0;
    const double bb[4] = {672.0, -168.0, 32.0, -3.0};
    for (int n = 0; n < 4; ++n) c.bb[n] = bb[n] * denom;
    denom = 1.0 / 2520.0;
    const double cc[5] = {1627.0, -473.0, 127.0, -23.0, 2.0};
    for (int n = 0; n < 5; ++n) c.cc[n] = cc[n] * denom;
    denom = 1.0 / 1260.0;
    const double dd[4] = {126.0, 84.0, 36.0, 9.0};
    for (int n = 0; n < 4; ++n) c.dd[n] = dd[n] * denom;
    c.dd[4] = denom;
    c.nw = 11;
    // the highest wall row's weights are the centred ones minus a correction
    // a, each lower row's those of the row above minus its own a
    const double a[4][11] = {
        {1.0 / 840.0, -1.0 / 63.0, 3.0 / 28.0, -4.0 / 7.0, -11.0 / 30.0, 6.0 / 5.0, -0.5, 4.0 / 21.0, -3.0 / 56.0,
         1.0 / 105.0, -1.0 / 1260.0},
        {-1.0 / 360.0, 1.0 / 24.0, -3.0 / 8.0, -319.0 / 420.0, 1.75, -21.0 / 20.0, 7.0 / 12.0, -0.25, 0.075,
         -1.0 / 72.0, 1.0 / 840.0},
        {1.0 / 90.0, -2.0 / 9.0, -341.0 / 280.0, 8.0 / 3.0, -7.0 / 3.0, 28.0 / 15.0, -7.0 / 6.0, 8.0 / 15.0,
         -1.0 / 6.0, 2.0 / 63.0, -1.0 / 360.0},
        {-0.1, -4609.0 / 2520.0, 4.5, -6.0, 7.0, -6.3, 21.0 * 0.2, -2.0, 9.0 / 14.0, -0.125, 1.0 / 90.0}};
    for (int n = 0; n < 11; ++n) {
      const double centred = n < 5 ? c.cc[4 - n] : (n < 10 ? c.cc[n - 5] : 0.0);
      c.cw[3][n] = n < 10 ? centred - a[0][n] : -a[0][n];
      for (int r = 2; r >= 0; --r) c.cw[r][n] = c.cw[r + 1][n] - a[3 - r][n];
    }
  } else {  // order 5: flux_num_dnc5.F90:89-118, rhs/coefnearbnd_7p.F (denom 1/60)
    c.order = 5;
    denom = 1.0 / 12.0;
    c.bb[0] = 8.0 * denom; c.bb[1] = -denom;
    denom = 1.0 / 60.0;
    c.cc[0] = 37.0 * denom; c.cc[1] = -8.0 * denom; c.cc[2] = denom;
    c.dd[0] = 10.0 * denom; c.dd[1] = 5.0 * denom; c.dd[2] = denom;
    c.nw = 5;
    const double w3[5] = {12.0, 77.0, -43.0, 17.0, -3.0}, w5[5] = {-3.0, 27.0, 47.0, -13.0, 2.0};
    for (int n = 0; n < 5; ++n) { c.cw[0][n] = w3[n] * denom; c.cw[1][n] = w5[n] * denom; }
  }
}

inline Coef make_coef(const Phys& p, int order = 5) {
  Coef c;
  c.cpprandtl = p.cp / p.prandtl;
  c.cvm1 = 1.0 / p.cv;
  c.ccross = (0.25 / 3.0) * 0.0625;
  c.betas = p.muref * (p.tref + p.cs) / (sqrt(p.tref) * p.tref);
  c.gam1 = p.gam - 1.0;
  c.c2fac = p.gam * p.rgaz;
  double denom = 1.0 / 12.0;
  c.b1 = 8.0 * denom; c.b2 = -denom;
  denom = 1.0 / 60.0;
  c.c1 = 37.0 * denom; c.c2 = -8.0 * denom; c.c3 = denom;
  c.d1 = 10.0 * denom; c.d2 = 5.0 * denom; c.d3 = denom;
  c.c5[0] = -3.0 * denom; c.c5[1] = 27.0 * denom; c.c5[2] = 47.0 * denom; c.c5[3] = -13.0 * denom; c.c5[4] = 2.0 * denom;
  c.c3w[0] = 12.0 * denom; c.c3w[1] = 77.0 * denom; c.c3w[2] = -43.0 * denom; c.c3w[3] = 17.0 * denom; c.c3w[4] = -3.0 * denom;
  c.ct0 = 1.125; c.ct1 = -0.125;
  c.k2 = p.k2; c.k4 = p.k4; c.s_suth = p.s_suth;
  c.wall = 1;
  set_stencils(c, order);
  return c;
}

// Grid extents and index helpers.  Fortran indices (i, j) with i in
// [1-gh, im+gh]; q = linear index into a padded cell array.
struct Ext {
  int im, jm, gh, ni, nj;
  size_t np;  // padded cells
  __host__ __device__ inline int cidx(int i, int j) const { return (i + gh - 1) + (j + gh - 1) * ni; }
  __host__ __device__ inline int nidx(int i, int j) const { return (i + gh - 1) + (j + gh - 1) * (ni + 1); }
  __host__ __device__ inline size_t nn() const { return (size_t)(ni + 1) * (nj + 1); }
};

inline Ext make_ext(int im, int jm, int gh) {
  Ext e; e.im = im; e.jm = jm; e.gh = gh; e.ni = im + 2 * gh; e.nj = jm + 2 * gh; e.np = (size_t)e.ni * e.nj;
  return e;
}

// Fields of the primitive scratch (pass 1)
enum PField {
  F_U = 0, F_V, F_W, F_T, F_P, F_MU, F_F2, F_F3, F_F4, F_F5, F_G2, F_G3, F_G4, F_G5,
  F_SR, F_SU, F_SV, F_SC,  // sqrt(rho) and sqrt(rho) * (u, v, c^2) for the Roe average
  F_NPRIM
};
// Fields of the interpolation scratch (passes 1b and 1c): QI and QJ for
// u v w T mu, then for u v w T the point values of the 4th-order viscous face
// gradients, each shared by two faces: C (3-point along i), D (3-point along
// j), EI (4-point across i-face rows), NJ (4-point across j-face columns)
enum QField { Q_I = 0, Q_J = 5, V_C = 10, V_D = 14, V_EI = 18, V_NJ = 22, Q_NQ = 26 };
// Fields of the gradient scratch of the adjoint's forward pass
enum GField { G_UX = 0, G_UY, G_VX, G_VY, G_NGRAD };
// Fields of the sensor scratch of the residual pass 2 (k2 != 0), per cell of
// the interior and its one-cell ghost ring: the pressure sensor along i and
// along j, the Ducros ratio, 10 vol div(u) and the sound speed
enum SField { S_KSI = 0, S_KSJ, S_DUC, S_ARG, S_CS, S_NSENS };

// State accessor: value array plus K tangent arrays (stride dstride).
template <class S> struct State;
template <> struct State<double> {
  const double* __restrict__ v;
  BCG_HD double operator()(size_t q) const { return __ldg(v + q); }
};
template <int K> struct State<DK<K>> {
  const double* __restrict__ v;
  const double* __restrict__ d;
  size_t dstride;
  BCG_HD DK<K> operator()(size_t q) const {
    DK<K> r; r.v = __ldg(v + q);
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = __ldg(d + (size_t)k * dstride + q);
    return r;
  }
};

// Scratch accessor: nf fields, each (K+1) planes of `plane` doubles.
template <class S>
struct Scratch {
  double* __restrict__ p;
  size_t plane;
  static constexpr int NP = NDir<S>::value + 1;
  BCG_HD S ld(int field, size_t q) const { return Planes<S>::ld(p + (size_t)field * NP * plane, plane, q); }
  BCG_HD void st(int field, size_t q, const S& x) const { Planes<S>::st(p + (size_t)field * NP * plane, plane, q, x); }
};

}  // namespace bcg
