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
//   pass 2  cell gradients of u and v (Ducros sensor), once per interior cell;
//   pass 3  every face flux once (i- and j-faces of node (i,j)), then the
//           balance differences them into the residual.
#pragma once
#include "dual.cuh"

namespace bcg {

struct Phys {
  double cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4;
};

// scalar coefficients derived once on the host (flux_num_dnc5.f90:69-122, 938-950)
struct Coef {
  double cpprandtl, cvm1, ccross, betas, gam1, c2fac;  // c2fac = gam*rgaz
  double b1, b2, c1, c2, c3, d1, d2, d3;
  double c5[5], c3w[5];
  double ct0, ct1, k2, k4, s_suth;
  int wall;  // 1: adiabatic wall at j = 1 (flux_num_dnc5_2d); 0: centred rows everywhere (flux_num_dnc5_nowall_2d)
};

inline Coef make_coef(const Phys& p) {
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
// Fields of the gradient scratch (pass 2)
enum GField { G_UX = 0, G_UY, G_VX, G_VY, G_NGRAD };

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
