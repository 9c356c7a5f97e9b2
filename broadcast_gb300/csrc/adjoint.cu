// Adjoint (vector-Jacobian product) of the DNC5 residual for sm_103a.
//
// Reference: srcfv/adjoint/flux_num_dnc5_b.f90:15-6676 (Tapenade reverse mode
// of srcfv/prepro/flux_num_dnc5.f90): wb = (dR/dw)^T residub over every padded
// cell; wb is overwritten and the interior of residub is zeroed on return.
//
// Deterministic gather form, no atomics, three passes after the primal
// primitives (and gradients when k2 != 0):
//   1. k_adj_faces : per node, the i- and j-face fluxes are recomputed and
//      reversed; each face writes a record of 60 adjoint coefficients (Euler
//      and predictor line weights, Roe-average and sensor adjoints, viscous
//      point adjoints).  Nonlinear reverse work happens here, once per face.
//   2. k_adj_gather: per padded cell, the transposed stencils of all faces
//      that read the cell are applied to the records (linear, fixed
//      coefficients), giving the adjoints of the cell primitives, the direct
//      adjoints of w, and the adjoints of the 4th-order velocity gradients.
//   3. k_adj_final : per padded cell, the transposed gradient stencil and the
//      reverse of the primitive map give wb; residub's interior is zeroed.
#include "dnc5.cuh"
#include "residual.h"
#include "residual_impl.cuh"
#include "adjoint.h"

namespace bcg {

// record layout (fields of NREC planes over the (im+1) x (jm+1) node set)
enum Rec {
  R_EA = 0,    // 5: hb_e * nx   (Euler f line weights)
  R_EB = 5,    // 5: hb_e * ny   (Euler g line weights)
  R_PR = 10,   // 5: predictor adjoint  -rspec*eps4*hb_e
  R_DF = 15,   // 5: half-difference adjoint -rspec*eps2*hb_e/2 (+R, -L)
  R_ROE = 20,  // 8: rho, rho u, rho v, T of L then R (spectral radius, dxm)
  R_SP = 28,   // 4: pressure at LL, L, R, RR (sensor); wall: p(i,1), p(i,2)
  R_SG = 32,   // 8: gradients (ux, uy, vx, vy) at L then R (sensor)
  R_VS = 40,   // 16: viscous point adjoints, variable (u,v,w,T) x (N,S,E,O); wall: u,v,w at 40..42
  R_VM = 56,   // 4: adjoints of uu, vv, ww, mmu (lambda folded into mmu)
  NREC = 60
};
constexpr int W_P1 = R_SP, W_P2 = R_SP + 1, W_U = R_VS, W_V = R_VS + 1, W_W = R_VS + 2, W_MU = R_VM + 3;

// per-cell adjoint scratch (after the gather)
enum CellAdj {
  A_U = 0, A_V, A_W, A_T, A_P, A_MU, A_F2, A_F3, A_F4, A_F5, A_G2, A_G3, A_G4, A_G5,  // primitive adjoints
  A_W1, A_W2, A_W3, A_W4, A_W5,                                                       // direct w adjoints
  A_GUI, A_GUJ, A_GVI, A_GVJ,                                                         // gradient-stencil adjoints
  NCADJ
};

// cotangent of a batched call: blockIdx.y (every kernel below runs one
// cotangent per grid row; its residub / wb planes are cstride doubles apart,
// its records and gathered adjoints kstride doubles apart in the scratch)
BCG_HD size_t ycot() {
#ifdef __CUDA_ARCH__
  return blockIdx.y;
#else
  return 0;
#endif
}

struct AdjCtx {
  Ext e;
  Coef c;
  const double* __restrict__ w;
  const double* __restrict__ pr;   // primitive scratch (F_* fields, np each)
  const double* __restrict__ gr;   // gradient scratch (G_* fields, np each)
  const double* __restrict__ qr;   // interpolation rows and point values of the forward passes (Q_*, V_* fields)
  const double* __restrict__ nx;
  const double* __restrict__ ny;
  const double* __restrict__ vol;
  const double* __restrict__ volf;
  const double* __restrict__ rb;   // residub (ni, nj, 5)
  double* __restrict__ rec1;       // i-face records NREC x nn
  double* __restrict__ rec2;       // j-face records
  size_t nn;                       // (im+1)(jm+1)
  size_t cstride;                  // doubles between the residub planes of consecutive cotangents
  size_t kstride;                  // doubles between the scratch blocks of consecutive cotangents

  BCG_HD double W(int i, int j, int v) const { return __ldg(w + (size_t)e.cidx(i, j) + (size_t)(v - 1) * e.np); }
  BCG_HD double P(int f, int i, int j) const { return __ldg(pr + (size_t)f * e.np + e.cidx(i, j)); }
  BCG_HD double Q(int f, int i, int j) const { return __ldg(qr + (size_t)f * e.np + e.cidx(i, j)); }
  BCG_HD double Gr(int f, int i, int j) const {
    auto g = [&](int ii, int jj) { return __ldg(gr + (size_t)f * e.np + e.cidx(ii, jj)); };
    if (i == 0) return 2.0 * g(1, j) - g(2, j);
    if (i == e.im + 1) return 2.0 * g(e.im, j) - g(e.im - 1, j);
    if (j == e.jm + 1) return 2.0 * g(i, e.jm) - g(i, e.jm - 1);
    if (j == 0) return 2.0 * g(i, 1) - g(i, 2);  // no-wall j-faces at j = 1
    return g(i, j);
  }
  BCG_HD double NX(int i, int j, int d) const { return __ldg(nx + (size_t)(d - 1) * e.nn() + e.nidx(i, j)); }
  BCG_HD double NY(int i, int j, int d) const { return __ldg(ny + (size_t)(d - 1) * e.nn() + e.nidx(i, j)); }
  BCG_HD double VOL(int i, int j) const { return __ldg(vol + e.cidx(i, j)); }
  BCG_HD double VOLF(int i, int j, int d) const { return __ldg(volf + (size_t)(d - 1) * e.np + e.cidx(i, j)); }
  BCG_HD double RB(int i, int j, int v) const {
    if (i < 1 || i > e.im || j < 1 || j > e.jm) return 0.0;
    return __ldg(rb + ycot() * cstride + (size_t)e.cidx(i, j) + (size_t)(v - 1) * e.np);
  }
  BCG_HD static double q4(double a, double b, double cc, double d) { return -a + 9.0 * b + 9.0 * cc - d; }
};

// reverse of the viscous flux formulas (rhs/flux_visqueux_o4_i.F:80-103):
// given fvb, gvb (adjoints of fv[0..3], gv[0..3]) and the forward values,
// accumulate adjoints of mmu, lambda, uu, vv, ww and of the 8 face gradients.
BCG_HD void visc_fluxes_rev(double mmu, double lambda, double uu, double vv, double ww, const double g[8],
                            const double fvb_in[4], const double gvb_in[4], double& mmub, double& lambdab,
                            double& uub, double& vvb, double& wwb, double gb[8]) {
  const double TWOTHIRD = 2.0 / 3.0;
  const double ux = g[0], uy = g[1], vx = g[2], vy = g[3], wx = g[4], wy = g[5], tx = g[6], ty = g[7];
  const double fv0 = TWOTHIRD * mmu * (2.0 * ux - vy), fv1 = mmu * (uy + vx), fv2 = mmu * wx;
  const double gv0 = mmu * (uy + vx), gv1 = TWOTHIRD * mmu * (-ux + 2.0 * vy), gv2 = mmu * wy;
  const double fv3b = fvb_in[3], gv3b = gvb_in[3];
  const double fv0b = fvb_in[0] + uu * fv3b, fv1b = fvb_in[1] + vv * fv3b, fv2b = fvb_in[2] + ww * fv3b;
  const double gv0b = gvb_in[0] + uu * gv3b, gv1b = gvb_in[1] + vv * gv3b, gv2b = gvb_in[2] + ww * gv3b;
  uub += fv0 * fv3b + gv0 * gv3b;
  vvb += fv1 * fv3b + gv1 * gv3b;
  wwb += fv2 * fv3b + gv2 * gv3b;
  lambdab += tx * fv3b + ty * gv3b;
  gb[6] += lambda * fv3b;
  gb[7] += lambda * gv3b;
  mmub += TWOTHIRD * (2.0 * ux - vy) * fv0b + (uy + vx) * (fv1b + gv0b) + wx * fv2b +
          TWOTHIRD * (-ux + 2.0 * vy) * gv1b + wy * gv2b;
  gb[0] += TWOTHIRD * mmu * (2.0 * fv0b - gv1b);
  gb[3] += TWOTHIRD * mmu * (-fv0b + 2.0 * gv1b);
  gb[1] += mmu * (fv1b + gv0b);
  gb[2] += mmu * (fv1b + gv0b);
  gb[4] += mmu * fv2b;
  gb[5] += mmu * gv2b;
}

// Forward pieces of one face needed by the reverse: the 4 point values of each
// viscous variable and the face gradient coefficients.
struct ViscPts {
  double val[4][4];  // variable (u,v,w,T) x point (N,S,E,O)
  double ax[4], ay[4];  // gradient coefficients nX*volm1 for N,S,E,O (x and y)
  double uu, vv, ww, mmu, lambda;
};

BCG_HD void visc_points_i(const AdjCtx& a, int i, int j, bool o2, ViscPts& v) {
  const double volm1 = a.VOLF(i, j, 1);
  const double nxN = 0.5 * (a.NX(i + 1, j, 1) + a.NX(i, j, 1)), nxS = -(0.5 * (a.NX(i - 1, j, 1) + a.NX(i, j, 1)));
  const double nxO = 0.5 * (a.NX(i - 1, j + 1, 2) + a.NX(i, j + 1, 2)), nxE = -(0.5 * (a.NX(i - 1, j, 2) + a.NX(i, j, 2)));
  const double nyN = 0.5 * (a.NY(i + 1, j, 1) + a.NY(i, j, 1)), nyS = -(0.5 * (a.NY(i - 1, j, 1) + a.NY(i, j, 1)));
  const double nyO = 0.5 * (a.NY(i - 1, j + 1, 2) + a.NY(i, j + 1, 2)), nyE = -(0.5 * (a.NY(i - 1, j, 2) + a.NY(i, j, 2)));
  v.ax[0] = nxN * volm1; v.ax[1] = nxS * volm1; v.ax[2] = nxE * volm1; v.ax[3] = nxO * volm1;
  v.ay[0] = nyN * volm1; v.ay[1] = nyS * volm1; v.ay[2] = nyE * volm1; v.ay[3] = nyO * volm1;
  const int fl[4] = {F_U, F_V, F_W, F_T};
  for (int q = 0; q < 4; ++q) {
    const int f = fl[q];
    if (!o2) {
      // the forward passes' 3-point values (V_C: 26 P(i) - (P(i+1) + P(i-1)))
      // and 4-point combinations of the interpolation rows (V_EI), with the
      // stencils' constant factors
      const double T24 = 1.0 / 24.0, cc = a.c.ccross;
      v.val[q][0] = T24 * a.Q(V_C + q, i, j);
      v.val[q][1] = T24 * a.Q(V_C + q, i - 1, j);
      v.val[q][2] = cc * a.Q(V_EI + q, i, j);
      v.val[q][3] = cc * a.Q(V_EI + q, i, j + 1);
    } else {
      v.val[q][0] = a.P(f, i, j);
      v.val[q][1] = a.P(f, i - 1, j);
      v.val[q][2] = 0.25 * (a.P(f, i, j) + a.P(f, i, j - 1) + a.P(f, i - 1, j) + a.P(f, i - 1, j - 1));
      v.val[q][3] = 0.25 * (a.P(f, i, j) + a.P(f, i, j + 1) + a.P(f, i - 1, j) + a.P(f, i - 1, j + 1));
    }
  }
  if (!o2) {  // the interpolation rows QI at the face
    v.uu = 0.0625 * a.Q(Q_I + 0, i, j);
    v.vv = 0.0625 * a.Q(Q_I + 1, i, j);
    v.ww = 0.0625 * a.Q(Q_I + 2, i, j);
    v.mmu = 0.0625 * a.Q(Q_I + 4, i, j);
  } else {
    v.uu = 0.5 * (a.P(F_U, i, j) + a.P(F_U, i - 1, j));
    v.vv = 0.5 * (a.P(F_V, i, j) + a.P(F_V, i - 1, j));
    v.ww = 0.5 * (a.P(F_W, i, j) + a.P(F_W, i - 1, j));
    v.mmu = 0.5 * (a.P(F_MU, i, j) + a.P(F_MU, i - 1, j));
  }
  v.lambda = v.mmu * a.c.cpprandtl;
}

BCG_HD void visc_points_j(const AdjCtx& a, int i, int j, bool o2, ViscPts& v) {
  const double volm1 = a.VOLF(i, j, 2);
  const double nxN = 0.5 * (a.NX(i + 1, j - 1, 1) + a.NX(i + 1, j, 1)), nxS = -(0.5 * (a.NX(i, j - 1, 1) + a.NX(i, j, 1)));
  const double nxO = 0.5 * (a.NX(i, j + 1, 2) + a.NX(i, j, 2)), nxE = -(0.5 * (a.NX(i, j - 1, 2) + a.NX(i, j, 2)));
  const double nyN = 0.5 * (a.NY(i + 1, j - 1, 1) + a.NY(i + 1, j, 1)), nyS = -(0.5 * (a.NY(i, j - 1, 1) + a.NY(i, j, 1)));
  const double nyO = 0.5 * (a.NY(i, j + 1, 2) + a.NY(i, j, 2)), nyE = -(0.5 * (a.NY(i, j - 1, 2) + a.NY(i, j, 2)));
  v.ax[0] = nxN * volm1; v.ax[1] = nxS * volm1; v.ax[2] = nxE * volm1; v.ax[3] = nxO * volm1;
  v.ay[0] = nyN * volm1; v.ay[1] = nyS * volm1; v.ay[2] = nyE * volm1; v.ay[3] = nyO * volm1;
  const int fl[4] = {F_U, F_V, F_W, F_T};
  for (int q = 0; q < 4; ++q) {
    const int f = fl[q];
    if (!o2) {  // V_NJ: 4-point combinations of the rows QJ; V_D: 3-point values along j
      const double T24 = 1.0 / 24.0, cc = a.c.ccross;
      v.val[q][0] = cc * a.Q(V_NJ + q, i + 1, j);
      v.val[q][1] = cc * a.Q(V_NJ + q, i, j);
      v.val[q][2] = T24 * a.Q(V_D + q, i, j - 1);
      v.val[q][3] = T24 * a.Q(V_D + q, i, j);
    } else {
      v.val[q][0] = 0.25 * (a.P(f, i, j) + a.P(f, i + 1, j) + a.P(f, i, j - 1) + a.P(f, i + 1, j - 1));
      v.val[q][1] = 0.25 * (a.P(f, i, j) + a.P(f, i - 1, j) + a.P(f, i, j - 1) + a.P(f, i - 1, j - 1));
      v.val[q][2] = a.P(f, i, j - 1);
      v.val[q][3] = a.P(f, i, j);
    }
  }
  if (!o2) {  // the interpolation rows QJ at the face
    v.uu = 0.0625 * a.Q(Q_J + 0, i, j);
    v.vv = 0.0625 * a.Q(Q_J + 1, i, j);
    v.ww = 0.0625 * a.Q(Q_J + 2, i, j);
    v.mmu = 0.0625 * a.Q(Q_J + 4, i, j);
  } else {
    v.uu = 0.5 * (a.P(F_U, i, j) + a.P(F_U, i, j - 1));
    v.vv = 0.5 * (a.P(F_V, i, j) + a.P(F_V, i, j - 1));
    v.ww = 0.5 * (a.P(F_W, i, j) + a.P(F_W, i, j - 1));
    v.mmu = 0.5 * (a.P(F_MU, i, j) + a.P(F_MU, i, j - 1));
  }
  v.lambda = v.mmu * a.c.cpprandtl;
}

// One interior face (not the wall): reverse everything, write the record.
// dir 1: i-face (i,j) between L=(i-1,j) and R=(i,j); dir 2: j-face between
// L=(i,j-1) and R=(i,j).
BCG_HD void face_rev(const AdjCtx& a, int dir, int i, int j, double* __restrict__ rec, size_t nn, size_t slot) {
  const int iL = dir == 1 ? i - 1 : i, jL = dir == 1 ? j : j - 1;
  const int iLL = dir == 1 ? i - 2 : i, jLL = dir == 1 ? j : j - 2;
  const int iRR = dir == 1 ? i + 1 : i, jRR = dir == 1 ? j : j + 1;
  auto put = [&](int f, double x) { rec[(size_t)f * nn + slot] = x; };
  double hb[5];
  for (int v = 1; v <= 5; ++v) hb[v - 1] = a.RB(i, j, v) - a.RB(iL, jL, v);
  const double fnx = a.NX(i, j, dir), fny = a.NY(i, j, dir);
  // Euler: line weights
  for (int v = 0; v < 5; ++v) { put(R_EA + v, hb[v] * fnx); put(R_EB + v, hb[v] * fny); }
  // forward predictor and differences
  const int di = dir == 1 ? 1 : 0, dj = dir == 1 ? 0 : 1;
  double pred[5], diff[5];
  for (int v = 1; v <= 5; ++v) {
    auto ww = [&](int s) { return a.W(i + s * di, j + s * dj, v); };
    pred[v - 1] = -(a.c.d3 * ww(-3)) + a.c.d2 * ww(-2) - a.c.d1 * ww(-1) + a.c.d1 * ww(0) - a.c.d2 * ww(1) + a.c.d3 * ww(2);
    diff[v - 1] = 0.5 * (ww(0) - ww(-1));
  }
  // forward spectral radius (Roe average of L and R)
  const double rhomr = a.W(i, j, 1), rhoml = a.W(iL, jL, 1);
  // velocities of L and R from the primitives pass (rho u times the reciprocal of rho)
  const double ur = a.P(F_U, i, j), vr = a.P(F_V, i, j);
  const double ul = a.P(F_U, iL, jL), vl = a.P(F_V, iL, jL);
  const double c2r = a.c.c2fac * a.P(F_T, i, j), c2l = a.c.c2fac * a.P(F_T, iL, jL);
  const double qrat = rhomr / rhoml;
  const double rsq = (qrat == 0.0) ? 0.0 : rsqrt(qrat);  // r = sqrt(qrat) through rsqrt, reused by the reverse
  const double r = qrat * rsq;
  const double rr = 1.0 / (1.0 + r), omrr = 1.0 - rr;
  const double u = ul * rr + ur * omrr, v = vl * rr + vr * omrr;
  const double c2x = c2l * rr + c2r * omrr;
  const double nx2 = fnx * fnx + fny * fny;
  const double X = fnx * u + fny * v;
  const double c2n = c2x * nx2, rsc = (c2n == 0.0) ? 0.0 : rsqrt(c2n);
  const double sq = c2n * rsc;  // sqrt(c2x nx2) through rsqrt, reused by the reverse
  const double rspec = fabs(X) + sq;
  // forward sensor
  double eps2 = 0.0, eps4 = 0.0 < a.c.k4 ? a.c.k4 : 0.0;
  double ks1 = 0, ks2 = 0, A1 = 0, B1 = 0, A2 = 0, B2 = 0, du1 = 0, du2 = 0, dd1 = 0, dd2 = 0, vo1 = 0, vo2 = 0;
  double D1 = 0, D2 = 0, x1 = 0, x2 = 0, t1 = 0, t2 = 0, S1 = 0, S2 = 0, th1 = 0, th2 = 0, coef = 0, M1 = 0, M2 = 0,
         M3 = 0;
  const bool sensor = a.c.k2 != 0.0;
  if (sensor) {
    const double pL = a.P(F_P, iL, jL), pR = a.P(F_P, i, j), pLL = a.P(F_P, iLL, jLL), pRR = a.P(F_P, iRR, jRR);
    A1 = pL - 2.0 * pR + pRR; B1 = pL + 2.0 * pR + pRR;
    A2 = pLL - 2.0 * pL + pR; B2 = pLL + 2.0 * pL + pR;
    ks1 = fabs(A1) / fabs(B1);
    ks2 = fabs(A2) / fabs(B2);
    du1 = a.Gr(G_UX, i, j) + a.Gr(G_VY, i, j);
    vo1 = a.Gr(G_VX, i, j) - a.Gr(G_UY, i, j);
    D1 = du1 * du1 + vo1 * vo1 + 1e-15;
    dd1 = du1 * du1 / D1;
    S1 = sqrt(c2r * nx2);
    t1 = 10.0 * a.VOL(i, j) / (S1 + 1e-15);
    th1 = tanh(2.5 + t1 * du1);
    x1 = 0.5 * (1.0 - th1);
    du2 = a.Gr(G_UX, iL, jL) + a.Gr(G_VY, iL, jL);
    vo2 = a.Gr(G_VX, iL, jL) - a.Gr(G_UY, iL, jL);
    D2 = du2 * du2 + vo2 * vo2 + 1e-15;
    dd2 = du2 * du2 / D2;
    S2 = sqrt(c2l * nx2);
    t2 = 10.0 * a.VOL(iL, jL) / (S2 + 1e-15);
    th2 = tanh(2.5 + t2 * du2);
    x2 = 0.5 * (1.0 - th2);
    M1 = ks1 < ks2 ? ks2 : ks1;
    M2 = dd1 < dd2 ? dd2 : dd1;
    M3 = x1 < x2 ? x2 : x1;
    coef = M1 * M2 * M3;
    eps2 = a.c.k2 * coef;
    eps4 = 0.0 < a.c.k4 - eps2 * 12.0 ? a.c.k4 - eps2 * 12.0 : 0.0;
  }
  // ---- reverse of the dissipation: h -= rspec*(eps2*diff + eps4*pred)
  double rspecb = 0.0, eps2b = 0.0, eps4b = 0.0;
  for (int q = 0; q < 5; ++q) {
    const double db = -hb[q];
    rspecb += db * (eps2 * diff[q] + eps4 * pred[q]);
    eps2b += db * rspec * diff[q];
    eps4b += db * rspec * pred[q];
    put(R_PR + q, db * rspec * eps4);
    put(R_DF + q, 0.5 * db * rspec * eps2);
  }
  double rhoLb = 0, ruLb = 0, rvLb = 0, TLb = 0, rhoRb = 0, ruRb = 0, rvRb = 0, TRb = 0;
  double spb[4] = {0, 0, 0, 0}, sgb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (sensor) {
    if (0.0 < a.c.k4 - eps2 * 12.0) eps2b += -12.0 * eps4b;
    const double coefb = a.c.k2 * eps2b;
    const double M1b = coefb * M2 * M3, M2b = coefb * M1 * M3, M3b = coefb * M1 * M2;
    double ks1b = 0, ks2b = 0, dd1b = 0, dd2b = 0, x1b = 0, x2b = 0;
    if (ks1 < ks2) ks2b = M1b; else ks1b = M1b;
    if (dd1 < dd2) dd2b = M2b; else dd1b = M2b;
    if (x1 < x2) x2b = M3b; else x1b = M3b;
    // ks = |A|/|B|
    auto ksrev = [&](double ksb, double A, double B, double& Ab, double& Bb) {
      const double aB = fabs(B), aA = fabs(A);
      const double aAb = ksb / aB, aBb = -ksb * aA / (aB * aB);
      Ab = A >= 0.0 ? aAb : -aAb;
      Bb = B >= 0.0 ? aBb : -aBb;
    };
    double A1b, B1b, A2b, B2b;
    ksrev(ks1b, A1, B1, A1b, B1b);
    ksrev(ks2b, A2, B2, A2b, B2b);
    // A1,B1 over (L, R, RR); A2, B2 over (LL, L, R)
    spb[0] += A2b + B2b;                                  // LL
    spb[1] += A1b + B1b - 2.0 * A2b + 2.0 * B2b;          // L
    spb[2] += -2.0 * A1b + 2.0 * B1b + A2b + B2b;          // R
    spb[3] += A1b + B1b;                                  // RR
    // ducros and dxm of R (1) and L (2)
    auto side = [&](double ddb, double xb, double du, double vo, double D, double t, double S, double th, double c2,
                    double& dub, double& vob, double& c2b) {
      const double divu2b = ddb * (vo * vo + 1e-15) / (D * D);
      const double vort2b = -ddb * du * du / (D * D);
      dub = 2.0 * du * divu2b;
      vob = 2.0 * vo * vort2b;
      const double argb = -0.5 * (1.0 - th * th) * xb;
      dub += t * argb;
      const double tb = du * argb;
      const double Sb = -t / (S + 1e-15) * tb;
      c2b = (c2 * nx2 == 0.0) ? 0.0 : Sb * nx2 / (2.0 * S);
    };
    double du1b, vo1b, c2r_s, du2b, vo2b, c2l_s;
    side(dd1b, x1b, du1, vo1, D1, t1, S1, th1, c2r, du1b, vo1b, c2r_s);
    side(dd2b, x2b, du2, vo2, D2, t2, S2, th2, c2l, du2b, vo2b, c2l_s);
    // divu = ux + vy, vo = vx - uy   (order ux, uy, vx, vy)
    sgb[0] += du2b; sgb[1] -= vo2b; sgb[2] += vo2b; sgb[3] += du2b;  // L
    sgb[4] += du1b; sgb[5] -= vo1b; sgb[6] += vo1b; sgb[7] += du1b;  // R
    TRb += a.c.c2fac * c2r_s;
    TLb += a.c.c2fac * c2l_s;
  }
  // reverse of rspec = |X| + sqrt(c2x nx2) with the Roe average
  {
    const double Xb = X >= 0.0 ? rspecb : -rspecb;
    const double c2xb = rspecb * nx2 * (0.5 * rsc);
    const double ub = fnx * Xb, vb = fny * Xb;
    double rrb = ul * ub + vl * vb + c2l * c2xb;
    const double omrrb = ur * ub + vr * vb + c2r * c2xb;
    const double ulb = rr * ub, urb = omrr * ub, vlb = rr * vb, vrb = omrr * vb;
    const double c2lb = rr * c2xb, c2rb = omrr * c2xb;
    rrb -= omrrb;
    const double rb_ = -rr * rr * rrb;
    const double qb = rb_ * (0.5 * rsq);
    // the reverse divides by the two densities through their reciprocals
    const double irl = 1.0 / rhoml, irr = 1.0 / rhomr;
    rhoRb += qb * irl;
    rhoLb -= qb * qrat * irl;
    ruRb += urb * irr; rhoRb -= urb * ur * irr;
    rvRb += vrb * irr; rhoRb -= vrb * vr * irr;
    ruLb += ulb * irl; rhoLb -= ulb * ul * irl;
    rvLb += vlb * irl; rhoLb -= vlb * vl * irl;
    TRb += a.c.c2fac * c2rb;
    TLb += a.c.c2fac * c2lb;
  }
  put(R_ROE + 0, rhoLb); put(R_ROE + 1, ruLb); put(R_ROE + 2, rvLb); put(R_ROE + 3, TLb);
  put(R_ROE + 4, rhoRb); put(R_ROE + 5, ruRb); put(R_ROE + 6, rvRb); put(R_ROE + 7, TRb);
  for (int k = 0; k < 4; ++k) put(R_SP + k, spb[k]);
  for (int k = 0; k < 8; ++k) put(R_SG + k, sgb[k]);
  // ---- viscous: h_e -= (fv nxloc + gv nyloc) sn, e = 2..5
  const bool o2 = a.c.wall && ((dir == 1) ? (j <= 2) : (j == 2));
  ViscPts vp;
  if (dir == 1) visc_points_i(a, i, j, o2, vp); else visc_points_j(a, i, j, o2, vp);
  double g8[8];
  for (int q = 0; q < 4; ++q) {
    g8[2 * q] = vp.val[q][0] * vp.ax[0] + vp.val[q][1] * vp.ax[1] + vp.val[q][3] * vp.ax[3] + vp.val[q][2] * vp.ax[2];
    g8[2 * q + 1] = vp.val[q][0] * vp.ay[0] + vp.val[q][1] * vp.ay[1] + vp.val[q][3] * vp.ay[3] + vp.val[q][2] * vp.ay[2];
  }
  // (fv nx/|n| + gv ny/|n|) |n| = fv nx + gv ny (rhs/fluxnumassembly_i.F), as in the forward faces
  double fvb[4], gvb[4];
  for (int q = 0; q < 4; ++q) { fvb[q] = -hb[q + 1] * fnx; gvb[q] = -hb[q + 1] * fny; }
  double mmub = 0, lambdab = 0, uub = 0, vvb = 0, wwb = 0, gb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  visc_fluxes_rev(vp.mmu, vp.lambda, vp.uu, vp.vv, vp.ww, g8, fvb, gvb, mmub, lambdab, uub, vvb, wwb, gb);
  mmub += a.c.cpprandtl * lambdab;
  for (int q = 0; q < 4; ++q)
    for (int p = 0; p < 4; ++p) put(R_VS + 4 * q + p, vp.ax[p] * gb[2 * q] + vp.ay[p] * gb[2 * q + 1]);
  put(R_VM + 0, uub); put(R_VM + 1, vvb); put(R_VM + 2, wwb); put(R_VM + 3, mmub);
}

// adiabatic wall face (i,1) (rhs/fluxwall.F)
BCG_HD void wall_rev(const AdjCtx& a, int i, double* __restrict__ rec, size_t nn, size_t slot) {
  auto put = [&](int f, double x) { rec[(size_t)f * nn + slot] = x; };
  for (int f = 0; f < NREC; ++f) put(f, 0.0);
  const int j = 1;
  const double hb2 = a.RB(i, j, 2) - a.RB(i, j - 1, 2), hb3 = a.RB(i, j, 3) - a.RB(i, j - 1, 3);
  const double hb4 = a.RB(i, j, 4) - a.RB(i, j - 1, 4);
  const double nx2 = a.NX(i, j, 2), ny2 = a.NY(i, j, 2), vf = a.VOLF(i, j, 2);
  const double mmu = a.P(F_MU, i, j);
  const double u = a.P(F_U, i, j), v = a.P(F_V, i, j), w = a.P(F_W, i, j);
  const double ux = 2.0 * u * nx2 * vf, vx = 2.0 * v * nx2 * vf, wx = 2.0 * w * nx2 * vf;
  const double uy = 2.0 * u * ny2 * vf, vy = 2.0 * v * ny2 * vf, wy = 2.0 * w * ny2 * vf;
  const double TWOTHIRD = 2.0 / 3.0;
  const double pwb = hb2 * nx2 + hb3 * ny2;
  const double fvroub = -hb2 * nx2, gvroub = -hb2 * ny2, fvrovb = -hb3 * nx2, gvrovb = -hb3 * ny2;
  const double fvrowb = -hb4 * nx2, gvrowb = -hb4 * ny2;
  const double mmub = TWOTHIRD * (2.0 * ux - vy) * fvroub + (uy + vx) * (fvrovb + gvroub) + wx * fvrowb +
                      TWOTHIRD * (-ux + 2.0 * vy) * gvrovb + wy * gvrowb;
  const double uxb = TWOTHIRD * mmu * (2.0 * fvroub - gvrovb), vyb = TWOTHIRD * mmu * (-fvroub + 2.0 * gvrovb);
  const double uyb = mmu * (fvrovb + gvroub), vxb = uyb, wxb = mmu * fvrowb, wyb = mmu * gvrowb;
  put(W_P1, a.c.ct0 * pwb);
  put(W_P2, a.c.ct1 * pwb);
  put(W_MU, mmub);
  put(W_U, 2.0 * vf * (nx2 * uxb + ny2 * uyb));
  put(W_V, 2.0 * vf * (nx2 * vxb + ny2 * vyb));
  put(W_W, 2.0 * vf * (nx2 * wxb + ny2 * wyb));
}

__global__ void __launch_bounds__(128) k_adj_faces(AdjCtx a) {
  const Ext& e = a.e;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nI = e.im + 1;
  if (t >= nI * (e.jm + 1)) return;
  const int i = 1 + t % nI, j = 1 + t / nI;
  double* rec1 = a.rec1 + ycot() * a.kstride;
  double* rec2 = a.rec2 + ycot() * a.kstride;
  if (j <= e.jm) face_rev(a, 1, i, j, rec1, a.nn, t);
  if (i <= e.im) {
    if (j == 1 && a.c.wall) wall_rev(a, i, rec2, a.nn, t);
    else face_rev(a, 2, i, j, rec2, a.nn, t);
  }
}

// ---------------------------------------------------------------------------
// Gather: adjoint of every primitive of cell (ci, cj) from the records of the
// faces that read it.
struct GatherCtx {
  Ext e;
  Coef c;
  const double* __restrict__ rec1;
  const double* __restrict__ rec2;
  size_t nn;
  const double* __restrict__ nx;
  const double* __restrict__ ny;
  const double* __restrict__ vol;
  double* __restrict__ cadj;  // NCADJ x np
  size_t kstride;             // doubles between the scratch blocks of consecutive cotangents
  // cross-point weights (ccross * (-1, 9, 9, -1)[a]) * (-1, 7, 7, -1)[b], formed once on the host
  double wt[4][4];
  BCG_HD bool ifx(int i, int j) const { return i >= 1 && i <= e.im + 1 && j >= 1 && j <= e.jm; }
  BCG_HD bool jfx(int i, int j) const { return i >= 1 && i <= e.im && j >= 1 && j <= e.jm + 1; }
};

// weights of the line stencils, indexed by (cell - face) offset s in [-3, 2]
BCG_HD double w_euler(const Coef& c, int s) {
  switch (s) { case -3: return c.c3; case -2: return c.c2; case -1: return c.c1; case 0: return c.c1;
               case 1: return c.c2; case 2: return c.c3; default: return 0.0; }
}
BCG_HD double w_pred(const Coef& c, int s) {
  switch (s) { case -3: return -c.d3; case -2: return c.d2; case -1: return -c.d1; case 0: return c.d1;
               case 1: return -c.d2; case 2: return c.d3; default: return 0.0; }
}
BCG_HD double w_q4(int s) {  // -1 9 9 -1 over offsets -2..1
  switch (s) { case -2: return -1.0; case -1: return 9.0; case 0: return 9.0; case 1: return -1.0; default: return 0.0; }
}
BCG_HD double w_row(int s) {  // -1 7 7 -1 over offsets 0..3 from the first row
  switch (s) { case 0: return -1.0; case 1: return 7.0; case 2: return 7.0; case 3: return -1.0; default: return 0.0; }
}

// The viscous point adjoints of one face record (R_VS, R_VM) that reach a cell
// at offset (di, dj) = (cell - face) from the face, through the transposed
// point stencils: N and S are the face's own-direction 3-point values
// (T24 (-1, 26, -1)), E and O the cross points (ccross x the 4-point column
// (-1, 9, 9, -1) x the 4-point row (-1, 7, 7, -1)), uu..mmu the 4-point means
// (0.0625 (-1, 9, 9, -1)); the o2 rows (the wall's first rows) use 2-point
// and 4-cell averages.  Called from fully unrolled window loops, so di, dj
// and the zero pattern of the weights are constants and the zero terms drop
// out; the nonzero terms are summed in the order N, S, E, O.
template <bool IFACE, bool O2, class RF>
BCG_HD void gather_visc(const double (&wt)[4][4], int di, int dj, const RF& Rf, int i, int j, double ub[4],
                        double& mub) {
  const double T24 = 1.0 / 24.0;
  double cN = 0.0, cS = 0.0, cE = 0.0, cO = 0.0, cu = 0.0;  // integer stencil factors (0 = no term)
  bool xN = false, xS = false, xE = false, xO = false;      // factors that take ccross
  if constexpr (IFACE) {
    if constexpr (!O2) {
      cN = (dj == 0) ? (di == 1 ? -1.0 : di == 0 ? 26.0 : di == -1 ? -1.0 : 0.0) : 0.0;
      cS = (dj == 0) ? (di == 0 ? -1.0 : di == -1 ? 26.0 : di == -2 ? -1.0 : 0.0) : 0.0;
      const double col = w_q4(di);
      cE = col; cO = col;
      xE = w_row(dj + 2) != 0.0; xO = w_row(dj + 1) != 0.0;
      cu = (dj == 0) ? col : 0.0;
    } else {
      cN = (dj == 0 && di == 0) ? 1.0 : 0.0;
      cS = (dj == 0 && di == -1) ? 1.0 : 0.0;
      const bool col = (di == 0 || di == -1);
      cE = (col && (dj == 0 || dj == -1)) ? 1.0 : 0.0;
      cO = (col && (dj == 0 || dj == 1)) ? 1.0 : 0.0;
      cu = (col && dj == 0) ? 1.0 : 0.0;
    }
  } else {
    if constexpr (!O2) {
      const double row = w_q4(dj);
      cN = row; cS = row;
      xN = w_row(di + 1) != 0.0; xS = w_row(di + 2) != 0.0;
      cE = (di == 0) ? (dj == 0 ? -1.0 : dj == -1 ? 26.0 : dj == -2 ? -1.0 : 0.0) : 0.0;
      cO = (di == 0) ? (dj == 1 ? -1.0 : dj == 0 ? 26.0 : dj == -1 ? -1.0 : 0.0) : 0.0;
      cu = (di == 0) ? row : 0.0;
    } else {
      const bool rowok = (dj == 0 || dj == -1);
      cN = (rowok && (di == 0 || di == 1)) ? 1.0 : 0.0;
      cS = (rowok && (di == 0 || di == -1)) ? 1.0 : 0.0;
      cO = (di == 0 && dj == 0) ? 1.0 : 0.0;
      cE = (di == 0 && dj == -1) ? 1.0 : 0.0;
      cu = (di == 0 && rowok) ? 1.0 : 0.0;
    }
  }
  // the weights, in the forms (and roundings) of the point stencils
  double wN, wS, wE, wO, wuu;
  if constexpr (IFACE) {
    if constexpr (!O2) {
      wN = T24 * cN; wS = T24 * cS;
      wE = 0.0; wO = 0.0;  // from the table below
      wuu = 0.0625 * cu;
    } else {
      wN = cN; wS = cS; wE = 0.25 * cE; wO = 0.25 * cO; wuu = 0.5 * cu;
    }
  } else {
    if constexpr (!O2) {
      wN = 0.0; wS = 0.0;  // from the table below
      wE = T24 * cE; wO = T24 * cO;
      wuu = 0.0625 * cu;
    } else {
      wN = 0.25 * cN; wS = 0.25 * cS; wE = cE; wO = cO; wuu = 0.5 * cu;
    }
  }
  const bool hN = cN != 0.0 && (IFACE || O2 || xN), hS = cS != 0.0 && (IFACE || O2 || xS);
  const bool hE = cE != 0.0 && (!IFACE || O2 || xE), hO = cO != 0.0 && (!IFACE || O2 || xO);
  // the cross-point weights from the table (the same products, formed once)
  if constexpr (!O2) {
    if constexpr (IFACE) {
      if (hE) wE = wt[di + 2][dj + 2];
      if (hO) wO = wt[di + 2][dj + 1];
    } else {
      if (hN) wN = wt[dj + 2][di + 1];
      if (hS) wS = wt[dj + 2][di + 2];
    }
  }
  const bool hu = cu != 0.0;
  if (!(hN || hS || hE || hO || hu)) return;
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    double acc = 0.0;
    bool any = false;
    auto add = [&](bool has, double wt, int f) {
      if (!has) return;
      const double x = wt * Rf(f, i, j);
      acc = any ? acc + x : x;
      any = true;
    };
    add(hN, wN, R_VS + 4 * v + 0);
    add(hS, wS, R_VS + 4 * v + 1);
    add(hE, wE, R_VS + 4 * v + 2);
    add(hO, wO, R_VS + 4 * v + 3);
    if (any) ub[v] += acc;
  }
  if (hu) {
    ub[0] += wuu * Rf(R_VM + 0, i, j);
    ub[1] += wuu * Rf(R_VM + 1, i, j);
    ub[2] += wuu * Rf(R_VM + 2, i, j);
    mub += wuu * Rf(R_VM + 3, i, j);
  }
}

__global__ void __launch_bounds__(128) k_adj_gather(GatherCtx g) {
  // this cotangent's records
  const double* __restrict__ rec1 = g.rec1 + ycot() * g.kstride;
  const double* __restrict__ rec2 = g.rec2 + ycot() * g.kstride;
  auto R1 = [&](int f, int i, int j) { return __ldg(rec1 + (size_t)f * g.nn + (i - 1) + (size_t)(j - 1) * (g.e.im + 1)); };
  auto R2 = [&](int f, int i, int j) { return __ldg(rec2 + (size_t)f * g.nn + (i - 1) + (size_t)(j - 1) * (g.e.im + 1)); };
  const Ext& e = g.e;
  const Coef& c = g.c;
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= e.np) return;
  const int ci = (int)(q % e.ni) + 1 - e.gh, cj = (int)(q / e.ni) + 1 - e.gh;
  double fb[5] = {0, 0, 0, 0, 0}, gb[5] = {0, 0, 0, 0, 0}, wb[5] = {0, 0, 0, 0, 0};
  double ub[4] = {0, 0, 0, 0};  // u, v, w, T
  double pb = 0.0, mub = 0.0;
  // ---- i-faces -------------------------------------------------------------
  // Euler and predictor on row cj: faces i = ci - s, s in [-3, 2]
  for (int s = -3; s <= 2; ++s) {
    const int i = ci - s;
    if (!g.ifx(i, cj)) continue;
    const double we = w_euler(c, s), wp = w_pred(c, s);
    for (int v = 0; v < 5; ++v) {
      fb[v] += we * R1(R_EA + v, i, cj);
      gb[v] += we * R1(R_EB + v, i, cj);
      wb[v] += wp * R1(R_PR + v, i, cj);
    }
  }
  // differences, Roe average, sensor pressure: faces (ci, cj) [cell = R] and (ci+1, cj) [cell = L]
  if (g.ifx(ci, cj)) {
    for (int v = 0; v < 5; ++v) wb[v] += R1(R_DF + v, ci, cj);
    wb[0] += R1(R_ROE + 4, ci, cj); wb[1] += R1(R_ROE + 5, ci, cj); wb[2] += R1(R_ROE + 6, ci, cj);
    ub[3] += R1(R_ROE + 7, ci, cj);
  }
  if (g.ifx(ci + 1, cj)) {
    for (int v = 0; v < 5; ++v) wb[v] -= R1(R_DF + v, ci + 1, cj);
    wb[0] += R1(R_ROE + 0, ci + 1, cj); wb[1] += R1(R_ROE + 1, ci + 1, cj); wb[2] += R1(R_ROE + 2, ci + 1, cj);
    ub[3] += R1(R_ROE + 3, ci + 1, cj);
  }
  if (c.k2 != 0.0) {  // pressure of the sensor: face i uses LL=i-2, L=i-1, R=i, RR=i+1
    for (int k = 0; k < 4; ++k) {
      const int i = ci + 2 - k;  // cell = i-2+k
      if (g.ifx(i, cj)) pb += R1(R_SP + k, i, cj);
    }
  }
  // viscous: i-faces (i, j) with i - ci in [-1, 2] and j - cj in [-2, 2]
#pragma unroll
  for (int jj = -2; jj <= 2; ++jj)
#pragma unroll
    for (int ii = -1; ii <= 2; ++ii) {
      const int i = ci + ii, j = cj + jj;
      if (!g.ifx(i, j)) continue;
      if (c.wall && j <= 2) gather_visc<true, true>(g.wt, -ii, -jj, R1, i, j, ub, mub);
      else gather_visc<true, false>(g.wt, -ii, -jj, R1, i, j, ub, mub);
    }
  // ---- j-faces -------------------------------------------------------------
  // Euler: generic faces j >= 4 over rows j-3..j+2; near-wall faces 2, 3 over
  // rows 1..5 (without the wall: generic faces from j = 1)
  const int jgen = c.wall ? 4 : 1, jfirst = c.wall ? 2 : 1;
  for (int s = -3; s <= 2; ++s) {
    const int j = cj - s;
    if (j < jgen || !g.jfx(ci, j)) continue;
    const double we = w_euler(c, s);
    for (int v = 0; v < 5; ++v) { fb[v] += we * R2(R_EA + v, ci, j); gb[v] += we * R2(R_EB + v, ci, j); }
  }
  if (c.wall && cj >= 1 && cj <= 5) {
    for (int j = 2; j <= 3; ++j) {
      if (!g.jfx(ci, j)) continue;
      const double we = (j == 3) ? c.c5[cj - 1] : c.c3w[cj - 1];
      for (int v = 0; v < 5; ++v) { fb[v] += we * R2(R_EA + v, ci, j); gb[v] += we * R2(R_EB + v, ci, j); }
    }
  }
  // predictor: all j-faces j >= 2 (j >= 1 without the wall)
  for (int s = -3; s <= 2; ++s) {
    const int j = cj - s;
    if (j < jfirst || !g.jfx(ci, j)) continue;
    const double wp = w_pred(c, s);
    for (int v = 0; v < 5; ++v) wb[v] += wp * R2(R_PR + v, ci, j);
  }
  if (cj >= jfirst && g.jfx(ci, cj)) {
    for (int v = 0; v < 5; ++v) wb[v] += R2(R_DF + v, ci, cj);
    wb[0] += R2(R_ROE + 4, ci, cj); wb[1] += R2(R_ROE + 5, ci, cj); wb[2] += R2(R_ROE + 6, ci, cj);
    ub[3] += R2(R_ROE + 7, ci, cj);
  }
  if (cj + 1 >= jfirst && g.jfx(ci, cj + 1)) {
    for (int v = 0; v < 5; ++v) wb[v] -= R2(R_DF + v, ci, cj + 1);
    wb[0] += R2(R_ROE + 0, ci, cj + 1); wb[1] += R2(R_ROE + 1, ci, cj + 1); wb[2] += R2(R_ROE + 2, ci, cj + 1);
    ub[3] += R2(R_ROE + 3, ci, cj + 1);
  }
  if (c.k2 != 0.0) {
    for (int k = 0; k < 4; ++k) {
      const int j = cj + 2 - k;
      if (j >= jfirst && g.jfx(ci, j)) pb += R2(R_SP + k, ci, j);
    }
  }
  // wall faces (i, 1): p(i,1), p(i,2), mu(i,1), u v w (i,1)
  if (c.wall && g.jfx(ci, 1)) {
    if (cj == 1) {
      pb += R2(W_P1, ci, 1);
      mub += R2(W_MU, ci, 1);
      ub[0] += R2(W_U, ci, 1); ub[1] += R2(W_V, ci, 1); ub[2] += R2(W_W, ci, 1);
    } else if (cj == 2) {
      pb += R2(W_P2, ci, 1);
    }
  }
  // viscous j-faces (i, j) with i - ci in [-2, 2] and j - cj in [-1, 2]
#pragma unroll
  for (int jj = -1; jj <= 2; ++jj)
#pragma unroll
    for (int ii = -2; ii <= 2; ++ii) {
      const int i = ci + ii, j = cj + jj;
      if (j < jfirst || !g.jfx(i, j)) continue;
      if (c.wall && j == 2) gather_visc<false, true>(g.wt, -ii, -jj, R2, i, j, ub, mub);
      else gather_visc<false, false>(g.wt, -ii, -jj, R2, i, j, ub, mub);
    }
  // ---- gradient adjoints (interior cells, sensor only) ----------------------
  double gsb[4] = {0, 0, 0, 0};  // ux, uy, vx, vy
  if (c.k2 != 0.0 && ci >= 1 && ci <= e.im && cj >= 1 && cj <= e.jm) {
    auto addg = [&](double s, const double* base, int f0, int i, int j, bool i_face) {
      for (int k = 0; k < 4; ++k) gsb[k] += s * (i_face ? R1(f0 + k, i, j) : R2(f0 + k, i, j));
      (void)base;
    };
    if (g.ifx(ci, cj)) addg(1.0, nullptr, R_SG + 4, ci, cj, true);        // as R
    if (g.ifx(ci + 1, cj)) addg(1.0, nullptr, R_SG + 0, ci + 1, cj, true);  // as L
    if (ci == 1) addg(2.0, nullptr, R_SG + 0, 1, cj, true);                 // ghost i = 0 extrapolated
    if (ci == 2) addg(-1.0, nullptr, R_SG + 0, 1, cj, true);
    if (ci == e.im) addg(2.0, nullptr, R_SG + 4, e.im + 1, cj, true);       // ghost i = im+1
    if (ci == e.im - 1) addg(-1.0, nullptr, R_SG + 4, e.im + 1, cj, true);
    if (cj >= jfirst) addg(1.0, nullptr, R_SG + 4, ci, cj, false);
    if (cj + 1 <= e.jm + 1 && cj + 1 >= jfirst) addg(1.0, nullptr, R_SG + 0, ci, cj + 1, false);
    if (!c.wall && cj == 1) addg(2.0, nullptr, R_SG + 0, ci, 1, false);   // ghost j = 0 extrapolated
    if (!c.wall && cj == 2) addg(-1.0, nullptr, R_SG + 0, ci, 1, false);
    if (cj == e.jm) addg(2.0, nullptr, R_SG + 4, ci, e.jm + 1, false);     // ghost j = jm+1
    if (cj == e.jm - 1) addg(-1.0, nullptr, R_SG + 4, ci, e.jm + 1, false);
  }
  // store
  double* o = g.cadj + ycot() * g.kstride;
  const size_t np = e.np;
  o[A_U * np + q] = ub[0]; o[A_V * np + q] = ub[1]; o[A_W * np + q] = ub[2]; o[A_T * np + q] = ub[3];
  o[A_P * np + q] = pb; o[A_MU * np + q] = mub;
  for (int v = 1; v < 5; ++v) { o[(A_F2 + v - 1) * np + q] = fb[v]; o[(A_G2 + v - 1) * np + q] = gb[v]; }
  // f1 = rho u and g1 = rho v enter the direct w adjoints
  wb[1] += fb[0];
  wb[2] += gb[0];
  for (int v = 0; v < 5; ++v) o[(A_W1 + v) * np + q] = wb[v];
  // gradient-stencil adjoints gui_b = dxm1 ux_b + dym1 uy_b, ... (gradient.F)
  double gi[4] = {0, 0, 0, 0};
  if (c.k2 != 0.0 && ci >= 1 && ci <= e.im && cj >= 1 && cj <= e.jm) {
    const size_t nn = e.nn();
    const int a = e.nidx(ci, cj);
    const double volm1 = 1.0 / __ldg(g.vol + q);
    const double dxm1 = 0.5 * (__ldg(g.nx + a) + __ldg(g.nx + a + 1)) * volm1;
    const double dxm2 = 0.5 * (__ldg(g.nx + nn + a) + __ldg(g.nx + nn + a + e.ni + 1)) * volm1;
    const double dym1 = 0.5 * (__ldg(g.ny + a) + __ldg(g.ny + a + 1)) * volm1;
    const double dym2 = 0.5 * (__ldg(g.ny + nn + a) + __ldg(g.ny + nn + a + e.ni + 1)) * volm1;
    gi[0] = dxm1 * gsb[0] + dym1 * gsb[1];  // gui
    gi[1] = dxm2 * gsb[0] + dym2 * gsb[1];  // guj
    gi[2] = dxm1 * gsb[2] + dym1 * gsb[3];  // gvi
    gi[3] = dxm2 * gsb[2] + dym2 * gsb[3];  // gvj
  }
  o[A_GUI * np + q] = gi[0]; o[A_GUJ * np + q] = gi[1]; o[A_GVI * np + q] = gi[2]; o[A_GVJ * np + q] = gi[3];
}

// Final: transposed gradient stencil, reverse of the primitive map, zero rb.
__global__ void __launch_bounds__(256) k_adj_final(Ext e, Coef c, const double* __restrict__ w,
                                                   const double* __restrict__ cadj0, double* __restrict__ wbo0,
                                                   double* __restrict__ rb0, size_t cstride, size_t kstride) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= e.np) return;
  const double* __restrict__ cadj = cadj0 + blockIdx.y * kstride;
  double* __restrict__ wbo = wbo0 + blockIdx.y * cstride;
  double* __restrict__ rb = rb0 + blockIdx.y * cstride;
  const size_t np = e.np;
  auto A = [&](int f, long long qq) { return __ldg(cadj + (size_t)f * np + (size_t)qq); };
  const int ci = (int)(q % e.ni) + 1 - e.gh, cj = (int)(q / e.ni) + 1 - e.gh;
  double ub = A(A_U, q), vb = A(A_V, q), wvb = A(A_W, q), tb = A(A_T, q), pb = A(A_P, q), mub = A(A_MU, q);
  if (c.k2 != 0.0) {
    // u(c) enters gui(c') for c' = c -+ 1, 2 and guj(c') for c' = c -+ ni, 2ni (interior c')
    auto GI = [&](int f, int ii, int jj) {
      if (ii < 1 || ii > e.im || jj < 1 || jj > e.jm) return 0.0;
      return A(f, e.cidx(ii, jj));
    };
    ub += c.b1 * (GI(A_GUI, ci - 1, cj) - GI(A_GUI, ci + 1, cj)) + c.b2 * (GI(A_GUI, ci - 2, cj) - GI(A_GUI, ci + 2, cj)) +
          c.b1 * (GI(A_GUJ, ci, cj - 1) - GI(A_GUJ, ci, cj + 1)) + c.b2 * (GI(A_GUJ, ci, cj - 2) - GI(A_GUJ, ci, cj + 2));
    vb += c.b1 * (GI(A_GVI, ci - 1, cj) - GI(A_GVI, ci + 1, cj)) + c.b2 * (GI(A_GVI, ci - 2, cj) - GI(A_GVI, ci + 2, cj)) +
          c.b1 * (GI(A_GVJ, ci, cj - 1) - GI(A_GVJ, ci, cj + 1)) + c.b2 * (GI(A_GVJ, ci, cj - 2) - GI(A_GVJ, ci, cj + 2));
  }
  // forward primitives
  const double ro = __ldg(w + q), ru = __ldg(w + q + np), rv = __ldg(w + q + 2 * np), rw = __ldg(w + q + 3 * np);
  const double re = __ldg(w + q + 4 * np);
  const double rom1 = 1.0 / ro;
  const double u = ru * rom1, v = rv * rom1, ww = rw * rom1;
  const double ec = 0.5 * (u * u + v * v + ww * ww);
  const double eloc = (re - ec * ro) * rom1;
  const double t = eloc * c.cvm1;
  const double p = c.gam1 * ro * eloc;
  const double htot = (re + p) * rom1;
  double rob = A(A_W1, q), rub = A(A_W2, q), rvb = A(A_W3, q), rwb = A(A_W4, q), reb = A(A_W5, q);
  // mu = betas t^1.5 / (t + s)
  if (t != 0.0) {
    const double st = sqrt(t), den = t + c.s_suth;
    tb += mub * c.betas * st * (0.5 * t + 1.5 * c.s_suth) / (den * den);
  } else {
    tb += 0.0;
  }
  const double f2b = A(A_F2, q), f3b = A(A_F3, q), f4b = A(A_F4, q), f5b = A(A_F5, q);
  const double g2b = A(A_G2, q), g3b = A(A_G3, q), g4b = A(A_G4, q), g5b = A(A_G5, q);
  rub += u * f2b + v * f3b + ww * f4b + htot * f5b;
  rvb += u * g2b + v * g3b + ww * g4b + htot * g5b;
  ub += ru * f2b + rv * g2b;
  vb += ru * f3b + rv * g3b;
  wvb += ru * f4b + rv * g4b;
  pb += f2b + g3b;
  const double htotb = ru * f5b + rv * g5b;
  reb += rom1 * htotb;
  pb += rom1 * htotb;
  double rom1b = (re + p) * htotb;
  rob += c.gam1 * eloc * pb;
  double elocb = c.gam1 * ro * pb + c.cvm1 * tb;
  reb += rom1 * elocb;
  const double ecb = -ro * rom1 * elocb;
  rob += -ec * rom1 * elocb;
  rom1b += (re - ec * ro) * elocb;
  ub += u * ecb; vb += v * ecb; wvb += ww * ecb;
  rub += rom1 * ub; rvb += rom1 * vb; rwb += rom1 * wvb;
  rom1b += ru * ub + rv * vb + rw * wvb;
  rob += -rom1 * rom1 * rom1b;
  wbo[q] = rob; wbo[q + np] = rub; wbo[q + 2 * np] = rvb; wbo[q + 3 * np] = rwb; wbo[q + 4 * np] = reb;
  if (ci >= 1 && ci <= e.im && cj >= 1 && cj <= e.jm)
    for (int k = 0; k < 5; ++k) rb[q + (size_t)k * np] = 0.0;
}

size_t adjoint_cotangent_doubles(int im, int jm, int gh) {
  const Ext e = make_ext(im, jm, gh);
  const size_t nn = (size_t)(im + 1) * (jm + 1);
  return (size_t)NCADJ * e.np + 2 * (size_t)NREC * nn;
}

size_t adjoint_scratch_doubles(int im, int jm, int gh, int ncot) {
  const Ext e = make_ext(im, jm, gh);
  return (size_t)(F_NPRIM + G_NGRAD + Q_NQ) * e.np +
         (size_t)(ncot > 1 ? ncot : 1) * adjoint_cotangent_doubles(im, jm, gh);
}

cudaError_t run_adjoint(const AdjointArgs& a, cudaStream_t st) {
  const Ext e = make_ext(a.im, a.jm, a.gh);
  Coef c = make_coef(a.phys);
  c.wall = a.nowall ? 0 : 1;
  const size_t nn = (size_t)(a.im + 1) * (a.jm + 1);
  double* pr = a.scratch;
  double* gr = pr + (size_t)F_NPRIM * e.np;
  double* qr = gr + (size_t)G_NGRAD * e.np;
  double* cadj = qr + (size_t)Q_NQ * e.np;
  double* rec1 = cadj + (size_t)NCADJ * e.np;
  double* rec2 = rec1 + (size_t)NREC * nn;
  const int B = 256;
  const unsigned ncot = a.ncot > 1 ? (unsigned)a.ncot : 1u;
  const size_t cstride = a.cstride ? a.cstride : (size_t)5 * e.np;
  const size_t kstride = adjoint_cotangent_doubles(a.im, a.jm, a.gh);
  launch_primal_passes(e, c, a.w, pr, gr, a.nx, a.ny, a.vol, st);  // shared by the cotangents
  // the viscous point values of the 4th-order rows, as the forward residual forms them
  {
    const GroupStride gs{0, 0};
    const unsigned gq = (unsigned)((e.np + B - 1) / B);
    k_qrows<double><<<gq, B, 0, st>>>(e, Scratch<double>{pr, e.np}, Scratch<double>{qr, e.np}, gs);
    k_vpts<double><<<gq, B, 0, st>>>(e, Scratch<double>{qr, e.np}, gs);
  }
  AdjCtx ac{e, c, a.w, pr, gr, qr, a.nx, a.ny, a.vol, a.volf, a.rb, rec1, rec2, nn, cstride, kstride};
  const int BF = 128;
  k_adj_faces<<<dim3((unsigned)((nn + BF - 1) / BF), ncot), BF, 0, st>>>(ac);
  GatherCtx gc{e, c, rec1, rec2, nn, a.nx, a.ny, a.vol, cadj, kstride, {}};
  const double q4w[4] = {-1.0, 9.0, 9.0, -1.0}, roww[4] = {-1.0, 7.0, 7.0, -1.0};
  for (int x = 0; x < 4; ++x)
    for (int y = 0; y < 4; ++y) gc.wt[x][y] = c.ccross * q4w[x] * roww[y];
  k_adj_gather<<<dim3((unsigned)((e.np + BF - 1) / BF), ncot), BF, 0, st>>>(gc);
  k_adj_final<<<dim3((unsigned)((e.np + B - 1) / B), ncot), B, 0, st>>>(e, c, a.w, cadj, a.wb, a.rb, cstride, kstride);
  return cudaGetLastError();
}

}  // namespace bcg
