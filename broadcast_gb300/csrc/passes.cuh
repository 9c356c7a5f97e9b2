// Per-element bodies of the DNC5 residual passes, written over a scalar type S
// (double, or DK<K> for the fused residual + K-direction JVP).  Included by
// the single-grid kernels (residual.cu) and the uneven-batch kernels
// (batch.cu), which differ only in how a thread finds its grid and element.
//
// Reference: srcfv/prepro/flux_num_dnc5.f90 (flattened
// srcfv/rhs/flux_num_dnc5.F90 with its rhs/ and phys/ fragments).
#pragma once
#include "dnc5.cuh"

namespace bcg {

// ---------------------------------------------------------------------------
// pass 1: primitives on padded cell q (phys/Primitives.F, phys/viscosity.F)
template <class S>
BCG_HD void prim_cell(const Ext& e, const Coef& c, const State<S>& w, const Scratch<S>& pr, size_t q) {
  const size_t n = e.np;
  const S ro = w(q), ru = w(q + n), rv = w(q + 2 * n), rw = w(q + 3 * n), re = w(q + 4 * n);
  const S rom1 = 1.0 / ro;
  const S u = ru * rom1, v = rv * rom1, ww = rw * rom1;
  // energies and pressure rounded operation by operation in the reference's
  // order: the pressure sensor's MAX/abs branches follow the pressure's bits
  const S ec = 0.5 * add_rn(add_rn(mul_rn(u, u), mul_rn(v, v)), mul_rn(ww, ww));
  const S eloc = mul_rn(sub_rn(re, mul_rn(ec, ro)), rom1);
  const S t = eloc * c.cvm1;
  const S p = mul_rn(mul_rn(c.gam1, ro), eloc);
  const S htot = (re + p) * rom1;
  pr.st(F_U, q, u); pr.st(F_V, q, v); pr.st(F_W, q, ww); pr.st(F_T, q, t); pr.st(F_P, q, p);
  pr.st(F_F2, q, ru * u + p); pr.st(F_F3, q, ru * v); pr.st(F_F4, q, ru * ww); pr.st(F_F5, q, ru * htot);
  pr.st(F_G2, q, rv * u); pr.st(F_G3, q, rv * v + p); pr.st(F_G4, q, rv * ww); pr.st(F_G5, q, rv * htot);
  pr.st(F_MU, q, c.betas / (t + c.s_suth) * sqrt_r(t) * t);
  // Roe-average ingredients: sqrt(rho), and sqrt(rho) times u, v and c^2
  const S sr = sqrt_r(ro);
  pr.st(F_SR, q, sr);
  pr.st(F_SU, q, sr * u);
  pr.st(F_SV, q, sr * v);
  pr.st(F_SC, q, sr * (c.c2fac * t));
}

// ---------------------------------------------------------------------------
// pass 1b: the 4-point interpolations (-a + 9b + 9c - d) that the 4th-order
// viscous fluxes read, once per face location instead of once per face use:
//   QI at i-face location (i, j): cells i-2..i+1 of row j,  i in [1, im+1], j in [-1, jm+2]
//   QJ at j-face location (i, j): rows j-2..j+1 of column i, i in [-1, im+2], j in [2, jm+1]
// for u, v, w, T and mu (rhs/flux_visqueux_o4_i.F, _j.F).
template <class S>
BCG_HD void qrows_cell(const Ext& e, const Scratch<S>& pr, const Scratch<S>& qr, size_t q) {
  const int i = (int)(q % e.ni) + 1 - e.gh, j = (int)(q / e.ni) + 1 - e.gh;
  const int fl[5] = {F_U, F_V, F_W, F_T, F_MU};
  const int di = 1, dj = e.ni;
  if (i >= 1 && i <= e.im + 1 && j >= -1 && j <= e.jm + 2) {
#pragma unroll
    for (int a = 0; a < 5; ++a) {
      const S x0 = pr.ld(fl[a], q - 2 * di), x1 = pr.ld(fl[a], q - di), x2 = pr.ld(fl[a], q), x3 = pr.ld(fl[a], q + di);
      qr.st(Q_I + a, q, 9.0 * (x1 + x2) - (x0 + x3));
    }
  }
  if (i >= -1 && i <= e.im + 2 && j >= 1 && j <= e.jm + 1) {
#pragma unroll
    for (int a = 0; a < 5; ++a) {
      const S x0 = pr.ld(fl[a], q - 2 * dj), x1 = pr.ld(fl[a], q - dj), x2 = pr.ld(fl[a], q), x3 = pr.ld(fl[a], q + dj);
      qr.st(Q_J + a, q, 9.0 * (x1 + x2) - (x0 + x3));
    }
  }
  // 3-point values 26 q(c) - (q(c+1) + q(c-1)) of u v w T:
  //   C along i at i in [0, im+1], j in [1, jm]   (i-faces (i,j), (i+1,j))
  //   D along j at i in [1, im], j in [0, jm+1]   (j-faces (i,j), (i,j+1))
  // (the wall rows use only j >= 3 and j >= 2 of them; without a wall all rows are centred)
  if (i >= 0 && i <= e.im + 1 && j >= 1 && j <= e.jm) {
#pragma unroll
    for (int a = 0; a < 4; ++a)
      qr.st(V_C + a, q, 26.0 * pr.ld(fl[a], q) - (pr.ld(fl[a], q + di) + pr.ld(fl[a], q - di)));
  }
  if (i >= 1 && i <= e.im && j >= 0 && j <= e.jm + 1) {
#pragma unroll
    for (int a = 0; a < 4; ++a)
      qr.st(V_D + a, q, 26.0 * pr.ld(fl[a], q) - (pr.ld(fl[a], q + dj) + pr.ld(fl[a], q - dj)));
  }
}

// pass 1c: the 4-point combinations 7 (b + c) - (a + d) of the interpolation
// rows, at i in [1, im+1], j in [1, jm+1]:
//   EI(i,j) from QI(i, j-2..j+1)  (vE / vO of the i-faces (i,j) / (i,j-1))
//   NJ(i,j) from QJ(i-2..i+1, j)  (vS / vN of the j-faces (i,j) / (i-1,j))
template <class S>
BCG_HD void vpts_cell(const Ext& e, const Scratch<S>& qr, size_t q) {
  const int i = (int)(q % e.ni) + 1 - e.gh, j = (int)(q / e.ni) + 1 - e.gh;
  if (i < 1 || i > e.im + 1 || j < 1 || j > e.jm + 1) return;
  const int di = 1, dj = e.ni;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const S y0 = qr.ld(Q_I + a, q - 2 * dj), y1 = qr.ld(Q_I + a, q - dj), y2 = qr.ld(Q_I + a, q), y3 = qr.ld(Q_I + a, q + dj);
    qr.st(V_EI + a, q, 7.0 * (y1 + y2) - (y0 + y3));
    const S z0 = qr.ld(Q_J + a, q - 2 * di), z1 = qr.ld(Q_J + a, q - di), z2 = qr.ld(Q_J + a, q), z3 = qr.ld(Q_J + a, q + di);
    qr.st(V_NJ + a, q, 7.0 * (z1 + z2) - (z0 + z3));
  }
}

// ---------------------------------------------------------------------------
// pass 2: cell gradients of u and v on interior cell t (row-major over the
// im x jm interior) (rhs/gradop_5pi.F, gradop_5pj.F, gradient.F; the 3p, 7p and
// 9p operators for R = 2, 4, 5)
template <class S, int R = 3>
BCG_HD void grad_cell(const Ext& e, const Coef& c, const Scratch<S>& pr, const Scratch<S>& gr,
                      const double* __restrict__ nx, const double* __restrict__ ny, const double* __restrict__ vol,
                      int t) {
  const int i = 1 + t % e.im, j = 1 + t / e.im;
  const size_t q = e.cidx(i, j);
  const int di = 1, dj = e.ni;
  auto g4 = [&](int f, int s) {
    S g = c.bb[0] * (pr.ld(f, q + s) - pr.ld(f, q - s));
#pragma unroll
    for (int n = 2; n < R; ++n) g = g + c.bb[n - 1] * (pr.ld(f, q + n * s) - pr.ld(f, q - n * s));
    return g;
  };
  const S gui = g4(F_U, di), gvi = g4(F_V, di), guj = g4(F_U, dj), gvj = g4(F_V, dj);
  const size_t nn = e.nn();
  const int a = e.nidx(i, j);
  const double volm1 = 1.0 / __ldg(vol + q);
  const double dxm1 = 0.5 * (__ldg(nx + a) + __ldg(nx + a + 1)) * volm1;
  const double dxm2 = 0.5 * (__ldg(nx + nn + a) + __ldg(nx + nn + a + e.ni + 1)) * volm1;
  const double dym1 = 0.5 * (__ldg(ny + a) + __ldg(ny + a + 1)) * volm1;
  const double dym2 = 0.5 * (__ldg(ny + nn + a) + __ldg(ny + nn + a + e.ni + 1)) * volm1;
  gr.st(G_UX, q, dxm1 * gui + dxm2 * guj);
  gr.st(G_VX, q, dxm1 * gvi + dxm2 * gvj);
  gr.st(G_UY, q, dym1 * gui + dym2 * guj);
  gr.st(G_VY, q, dym1 * gvi + dym2 * gvj);
}

// ---------------------------------------------------------------------------
// pass 2 of the residual (k2 != 0): the cell quantities of the pressure/Ducros
// sensor (rhs/ducrosfordnc_i.F, _j.F), once per cell instead of once per face
// that reads them, on element t of the (im+2) x (jm+2) cells i in [0, im+1],
// j in [0, jm+1] without the corners (the cells the faces' sensor reads):
//   KSI, KSJ  |p(c-1) - 2 p(c) + p(c+1)| / |p(c-1) + 2 p(c) + p(c+1)| along i
//             (rows 1..jm) and along j (columns 1..im), rounded operation by
//             operation in the reference's order, so MAX(ks1, ks2) of a face
//             compares the reference's values
//   DUC       div(u)^2 / (div(u)^2 + rot(u)^2 + 1e-15)
//   ARG       10 vol div(u), CS sqrt(gam R T): the face's tanh argument is
//             2.5 + ARG / (CS |n| + 1e-15)
// The u, v gradients are the 4th-order cell gradients (rhs/gradop_5pi.F,
// gradop_5pj.F, gradient.F; 3p, 7p, 9p for R = 2, 4, 5), on the ghost ring
// extrapolated from the two nearest interior cells (rhs/gradveloingh.F).
template <class S, int R = 3>
BCG_HD void cell_gradient(const Ext& e, const Coef& c, const Scratch<S>& pr, const double* __restrict__ nx,
                          const double* __restrict__ ny, const double* __restrict__ vol, int i, int j, S g[4]) {
  const size_t q = e.cidx(i, j);
  const int di = 1, dj = e.ni;
  auto g4 = [&](int f, int s) {
    S x = c.bb[0] * (pr.ld(f, q + s) - pr.ld(f, q - s));
#pragma unroll
    for (int n = 2; n < R; ++n) x = x + c.bb[n - 1] * (pr.ld(f, q + n * s) - pr.ld(f, q - n * s));
    return x;
  };
  const S gui = g4(F_U, di), gvi = g4(F_V, di), guj = g4(F_U, dj), gvj = g4(F_V, dj);
  const size_t nn = e.nn();
  const int a = e.nidx(i, j);
  const double volm1 = 1.0 / __ldg(vol + q);
  const double dxm1 = 0.5 * (__ldg(nx + a) + __ldg(nx + a + 1)) * volm1;
  const double dxm2 = 0.5 * (__ldg(nx + nn + a) + __ldg(nx + nn + a + e.ni + 1)) * volm1;
  const double dym1 = 0.5 * (__ldg(ny + a) + __ldg(ny + a + 1)) * volm1;
  const double dym2 = 0.5 * (__ldg(ny + nn + a) + __ldg(ny + nn + a + e.ni + 1)) * volm1;
  g[G_UX] = dxm1 * gui + dxm2 * guj;
  g[G_VX] = dxm1 * gvi + dxm2 * gvj;
  g[G_UY] = dym1 * gui + dym2 * guj;
  g[G_VY] = dym1 * gvi + dym2 * gvj;
}

template <class S>
BCG_HD S pressure_ratio(const S& pm, const S& p0, const S& pp) {
  const S p02 = 2.0 * p0;  // exact
  return div_rn(fabs_t(add_rn(sub_rn(pm, p02), pp)), fabs_t(add_rn(add_rn(pm, p02), pp)));
}

template <class S, int R = 3>
BCG_HD void sensor_cell(const Ext& e, const Coef& c, const Scratch<S>& pr, const Scratch<S>& sg,
                        const double* __restrict__ nx, const double* __restrict__ ny, const double* __restrict__ vol,
                        int t) {
  const int i = t % (e.im + 2), j = t / (e.im + 2);
  const bool iring = (i == 0 || i == e.im + 1), jring = (j == 0 || j == e.jm + 1);
  if (iring && jring) return;
  S g[4];
  if (!iring && !jring) {
    cell_gradient<S, R>(e, c, pr, nx, ny, vol, i, j, g);
  } else {
    // ghost ring: 2 g(nearest interior) - g(next interior), as the faces' gradients
    int i1 = i, j1 = j, i2 = i, j2 = j;
    if (i == 0) { i1 = 1; i2 = 2; } else if (i == e.im + 1) { i1 = e.im; i2 = e.im - 1; }
    else if (j == e.jm + 1) { j1 = e.jm; j2 = e.jm - 1; } else { j1 = 1; j2 = 2; }
    S g1[4], g2[4];
    cell_gradient<S, R>(e, c, pr, nx, ny, vol, i1, j1, g1);
    cell_gradient<S, R>(e, c, pr, nx, ny, vol, i2, j2, g2);
#pragma unroll
    for (int k = 0; k < 4; ++k) g[k] = 2.0 * g1[k] - g2[k];
  }
  const size_t q = e.cidx(i, j);
  const S divu = g[G_UX] + g[G_VY], vo = g[G_VX] - g[G_UY];
  const S divu2 = divu * divu, vort2 = vo * vo;
  sg.st(S_DUC, q, divu2 / (divu2 + vort2 + 1e-15));
  sg.st(S_ARG, q, (10.0 * __ldg(vol + q)) * divu);
  sg.st(S_CS, q, sqrt_t(c.c2fac * pr.ld(F_T, q)));
  if (!jring) sg.st(S_KSI, q, pressure_ratio(pr.ld(F_P, q - 1), pr.ld(F_P, q), pr.ld(F_P, q + 1)));
  if (!iring)
    sg.st(S_KSJ, q, pressure_ratio(pr.ld(F_P, q - e.ni), pr.ld(F_P, q), pr.ld(F_P, q + e.ni)));
}

// ---------------------------------------------------------------------------
// pass 3: face fluxes of the DNC scheme with R point pairs (R = 3: DNC5)
// RECT: the grid is rectilinear, i.e. every i-face normal has ny = 0 and every
// j-face normal nx = 0 exactly (face_rectilinear, checked per grid by the
// caller).  The products with those zero components are then left out: the
// centred flux's g half on i-faces and f half on j-faces, half of the viscous
// weights, one product of the normal velocity, and the square root of |n|^2
// (sqrt of the rounded square of x is |x| in binary floating point).  The
// sums are the same sums of the same nonzero products (x + 0 y = x).
template <class S, int R = 3, bool RECT = false>
struct FaceCtx {
  // near-wall off-centred j-fluxes read the first NW cell rows
  static constexpr int NW = R == 2 ? 2 : (R == 3 ? 5 : (R == 4 ? 9 : 11));
  // DNC3 uses the 2nd-order viscous flux on every row (rhs/flux_visqueux_o2.F)
  static constexpr bool ALL_O2 = (R == 2);
  Ext e;
  Coef c;
  State<S> w;
  Scratch<S> pr, gr, qr;
  const double* __restrict__ nx;
  const double* __restrict__ ny;
  const double* __restrict__ vol;
  const double* __restrict__ volf;

  BCG_HD S W(int i, int j, int v) const { return w((size_t)e.cidx(i, j) + (size_t)(v - 1) * e.np); }
  BCG_HD S P(int f, int i, int j) const { return pr.ld(f, e.cidx(i, j)); }
  BCG_HD S Q(int f, int i, int j) const { return qr.ld(f, e.cidx(i, j)); }
  // Euler flux components f(.,.,v), g(.,.,v) with f1 = rho u, g1 = rho v
  BCG_HD S Fl(int v, int i, int j) const { return v == 1 ? W(i, j, 2) : P(F_F2 + v - 2, i, j); }
  BCG_HD S Gl(int v, int i, int j) const { return v == 1 ? W(i, j, 3) : P(F_G2 + v - 2, i, j); }
  BCG_HD double NX(int i, int j, int d) const { return __ldg(nx + (size_t)(d - 1) * e.nn() + e.nidx(i, j)); }
  BCG_HD double NY(int i, int j, int d) const { return __ldg(ny + (size_t)(d - 1) * e.nn() + e.nidx(i, j)); }
  BCG_HD double VOL(int i, int j) const { return __ldg(vol + e.cidx(i, j)); }
  BCG_HD double VOLF(int i, int j, int d) const { return __ldg(volf + (size_t)(d - 1) * e.np + e.cidx(i, j)); }
  // sensor quantities of pass 2 (cells of the interior and its ghost ring)
  BCG_HD S SG(int f, int i, int j) const { return gr.ld(f, e.cidx(i, j)); }
  BCG_HD static S q4(const S& a, const S& b, const S& cc, const S& d) { return -a + 9.0 * b + 9.0 * cc - d; }

  // Normal viscous flux fv * snx + gv * sny (the only combination the face
  // assembly uses, rhs/fluxnumassembly_i.F) from the point values v[a][p] of
  // u v w T (a) at the points N, S, O, E (p) whose gradient coefficients are
  // ax[p], ay[p] (ux = sum_p ax[p] u_p, uy = sum_p ay[p] u_p).  With the
  // viscous fluxes of rhs/flux_visqueux_o4_i.F
  //   fv = (2/3 mu (2ux - vy), mu (uy + vx), mu wx, lambda tx + uu fv0 + vv fv1 + ww fv2)
  //   gv = (mu (uy + vx), 2/3 mu (2vy - ux), mu wy, lambda ty + uu gv0 + vv gv1 + ww gv2)
  // the projections are linear in the point values with per-face scalar
  // weights, formed once per face:
  //   fn0 = mu sum_p [(4/3 ax snx + ay sny) u_p + (ax sny - 2/3 ay snx) v_p]
  //   fn1 = mu sum_p [(ay snx - 2/3 ax sny) u_p + (ax snx + 4/3 ay sny) v_p]
  //   fn2 = mu sum_p (ax snx + ay sny) w_p,  fn3 = lambda sum_p (ax snx + ay sny) T_p + uu fn0 + vv fn1 + ww fn2
  template <class PV>
  BCG_HD void visc_normal(const PV& val, const double ax[4], const double ay[4], double snx, double sny,
                          const S& mmu, const S& uu, const S& vv, const S& ww, S fn[4]) const {
    const double T3 = 1.0 / 3.0, TWOTHIRD = 2.0 / 3.0;
    S an, bn, wn, tn;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      const double xs = ax[p] * snx, ys = ay[p] * sny, xn = ax[p] * sny, yn = ay[p] * snx;
      const double e = xs + ys, c00 = e + T3 * xs, c11 = e + T3 * ys;
      const double c01 = xn - TWOTHIRD * yn, c10 = yn - TWOTHIRD * xn;
      const S u = val(0, p), v = val(1, p);
      if (p == 0) {
        an = c00 * u + c01 * v;
        bn = c10 * u + c11 * v;
        wn = e * val(2, p);
        tn = e * val(3, p);
      } else {
        an = an + c00 * u + c01 * v;
        bn = bn + c10 * u + c11 * v;
        wn = wn + e * val(2, p);
        tn = tn + e * val(3, p);
      }
    }
    fn[0] = mmu * an;
    fn[1] = mmu * bn;
    fn[2] = mmu * wn;
    fn[3] = (mmu * c.cpprandtl) * tn + uu * fn[0] + vv * fn[1] + ww * fn[2];
  }

  // Viscous flux through i-face (i,j): o4 (rhs/flux_visqueux_o4_i.F) or o2
  // (rows 1-2).  The face gradients are linear in four point values N, S, E,
  // O; the point stencils' constant factors (1/24, ccross, 1/4) and the face
  // volume are folded into the geometric coefficients, and the cross rows come
  // from the QI interpolations.
  BCG_HD void visc_i(int i, int j, bool o2, double snx, double sny, S fn[4]) const {
    const double volm1 = VOLF(i, j, 1);
    const double fN = o2 ? volm1 : volm1 / 24.0, fE = o2 ? 0.25 * volm1 : c.ccross * volm1;
    // point value of variable a (u v w T) at point p
    auto val = [&](int a, int p) -> S {
      const int f = F_U + a;  // F_U, F_V, F_W, F_T are consecutive
      if (!o2) {
        if (p == 0) return Q(V_C + a, i, j);
        if (p == 1) return Q(V_C + a, i - 1, j);
        if (p == 2) return Q(V_EI + a, i, j + 1);
        return Q(V_EI + a, i, j);
      }
      if (p == 0) return P(f, i, j);
      if (p == 1) return P(f, i - 1, j);
      if (p == 2) return (P(f, i, j) + P(f, i, j + 1)) + (P(f, i - 1, j) + P(f, i - 1, j + 1));
      return (P(f, i, j) + P(f, i, j - 1)) + (P(f, i - 1, j) + P(f, i - 1, j - 1));
    };
    auto means = [&](S& uu, S& vv, S& ww, S& mmu) {
      if (!o2) {
        uu = 0.0625 * Q(Q_I + 0, i, j);
        vv = 0.0625 * Q(Q_I + 1, i, j);
        ww = 0.0625 * Q(Q_I + 2, i, j);
        mmu = 0.0625 * Q(Q_I + 4, i, j);
      } else {
        uu = 0.5 * (P(F_U, i, j) + P(F_U, i - 1, j));
        vv = 0.5 * (P(F_V, i, j) + P(F_V, i - 1, j));
        ww = 0.5 * (P(F_W, i, j) + P(F_W, i - 1, j));
        mmu = 0.5 * (P(F_MU, i, j) + P(F_MU, i - 1, j));
      }
    };
    S uu, vv, ww, mmu;
    if constexpr (RECT) {
      // ay of N and S and ax of E and O are zero, and sny: of the weights of
      // visc_normal, N and S keep c00 = e + e/3, c11 = e (e = ax snx), E and O
      // keep c01 = -2/3 yn, c10 = yn (yn = ay snx)
      const double T3 = 1.0 / 3.0, TWOTHIRD = 2.0 / 3.0;
      const double x0 = (0.5 * (NX(i + 1, j, 1) + NX(i, j, 1)) * fN) * snx;
      const double x1 = (-(0.5 * (NX(i - 1, j, 1) + NX(i, j, 1))) * fN) * snx;
      const double y2 = (0.5 * (NY(i - 1, j + 1, 2) + NY(i, j + 1, 2)) * fE) * snx;
      const double y3 = (-(0.5 * (NY(i - 1, j, 2) + NY(i, j, 2))) * fE) * snx;
      means(uu, vv, ww, mmu);
      S an = (x0 + T3 * x0) * val(0, 0);
      an = an + (x1 + T3 * x1) * val(0, 1);
      an = an + (-(TWOTHIRD * y2)) * val(1, 2);
      an = an + (-(TWOTHIRD * y3)) * val(1, 3);
      S bn = x0 * val(1, 0);
      bn = bn + x1 * val(1, 1);
      bn = bn + y2 * val(0, 2);
      bn = bn + y3 * val(0, 3);
      const S wn = x0 * val(2, 0) + x1 * val(2, 1);
      const S tn = x0 * val(3, 0) + x1 * val(3, 1);
      fn[0] = mmu * an;
      fn[1] = mmu * bn;
      fn[2] = mmu * wn;
      fn[3] = (mmu * c.cpprandtl) * tn + uu * fn[0] + vv * fn[1] + ww * fn[2];
    } else {
      // points N, S, O, E
      const double ax[4] = {0.5 * (NX(i + 1, j, 1) + NX(i, j, 1)) * fN, -(0.5 * (NX(i - 1, j, 1) + NX(i, j, 1))) * fN,
                            0.5 * (NX(i - 1, j + 1, 2) + NX(i, j + 1, 2)) * fE, -(0.5 * (NX(i - 1, j, 2) + NX(i, j, 2))) * fE};
      const double ay[4] = {0.5 * (NY(i + 1, j, 1) + NY(i, j, 1)) * fN, -(0.5 * (NY(i - 1, j, 1) + NY(i, j, 1))) * fN,
                            0.5 * (NY(i - 1, j + 1, 2) + NY(i, j + 1, 2)) * fE, -(0.5 * (NY(i - 1, j, 2) + NY(i, j, 2))) * fE};
      means(uu, vv, ww, mmu);
      visc_normal(val, ax, ay, snx, sny, mmu, uu, vv, ww, fn);
    }
  }

  // Viscous flux through j-face (i,j): o4 (rhs/flux_visqueux_o4_j.F) or o2 (row 2).
  BCG_HD void visc_j(int i, int j, bool o2, double snx, double sny, S fn[4]) const {
    const double volm1 = VOLF(i, j, 2);
    const double fN = o2 ? 0.25 * volm1 : c.ccross * volm1, fE = o2 ? volm1 : volm1 / 24.0;
    auto val = [&](int a, int p) -> S {
      const int f = F_U + a;  // F_U, F_V, F_W, F_T are consecutive
      if (!o2) {
        if (p == 0) return Q(V_NJ + a, i + 1, j);
        if (p == 1) return Q(V_NJ + a, i, j);
        if (p == 2) return Q(V_D + a, i, j);
        return Q(V_D + a, i, j - 1);
      }
      if (p == 0) return (P(f, i, j) + P(f, i + 1, j)) + (P(f, i, j - 1) + P(f, i + 1, j - 1));
      if (p == 1) return (P(f, i, j) + P(f, i - 1, j)) + (P(f, i, j - 1) + P(f, i - 1, j - 1));
      if (p == 2) return P(f, i, j);
      return P(f, i, j - 1);
    };
    auto means = [&](S& uu, S& vv, S& ww, S& mmu) {
      if (!o2) {
        uu = 0.0625 * Q(Q_J + 0, i, j);
        vv = 0.0625 * Q(Q_J + 1, i, j);
        ww = 0.0625 * Q(Q_J + 2, i, j);
        mmu = 0.0625 * Q(Q_J + 4, i, j);
      } else {
        uu = 0.5 * (P(F_U, i, j) + P(F_U, i, j - 1));
        vv = 0.5 * (P(F_V, i, j) + P(F_V, i, j - 1));
        ww = 0.5 * (P(F_W, i, j) + P(F_W, i, j - 1));
        mmu = 0.5 * (P(F_MU, i, j) + P(F_MU, i, j - 1));
      }
    };
    S uu, vv, ww, mmu;
    if constexpr (RECT) {
      // ay of N and S and ax of E and O are zero, and snx: N and S keep
      // c01 = xn, c10 = -2/3 xn (xn = ax sny), E and O keep c00 = e,
      // c11 = e + e/3 (e = ay sny)
      const double T3 = 1.0 / 3.0, TWOTHIRD = 2.0 / 3.0;
      const double x0 = (0.5 * (NX(i + 1, j - 1, 1) + NX(i + 1, j, 1)) * fN) * sny;
      const double x1 = (-(0.5 * (NX(i, j - 1, 1) + NX(i, j, 1))) * fN) * sny;
      const double y2 = (0.5 * (NY(i, j + 1, 2) + NY(i, j, 2)) * fE) * sny;
      const double y3 = (-(0.5 * (NY(i, j - 1, 2) + NY(i, j, 2))) * fE) * sny;
      means(uu, vv, ww, mmu);
      S an = x0 * val(1, 0);
      an = an + x1 * val(1, 1);
      an = an + y2 * val(0, 2);
      an = an + y3 * val(0, 3);
      S bn = (-(TWOTHIRD * x0)) * val(0, 0);
      bn = bn + (-(TWOTHIRD * x1)) * val(0, 1);
      bn = bn + (y2 + T3 * y2) * val(1, 2);
      bn = bn + (y3 + T3 * y3) * val(1, 3);
      const S wn = y2 * val(2, 2) + y3 * val(2, 3);
      const S tn = y2 * val(3, 2) + y3 * val(3, 3);
      fn[0] = mmu * an;
      fn[1] = mmu * bn;
      fn[2] = mmu * wn;
      fn[3] = (mmu * c.cpprandtl) * tn + uu * fn[0] + vv * fn[1] + ww * fn[2];
    } else {
      // points N, S, O, E
      const double ax[4] = {0.5 * (NX(i + 1, j - 1, 1) + NX(i + 1, j, 1)) * fN, -(0.5 * (NX(i, j - 1, 1) + NX(i, j, 1))) * fN,
                            0.5 * (NX(i, j + 1, 2) + NX(i, j, 2)) * fE, -(0.5 * (NX(i, j - 1, 2) + NX(i, j, 2))) * fE};
      const double ay[4] = {0.5 * (NY(i + 1, j - 1, 1) + NY(i + 1, j, 1)) * fN, -(0.5 * (NY(i, j - 1, 1) + NY(i, j, 1))) * fN,
                            0.5 * (NY(i, j + 1, 2) + NY(i, j, 2)) * fE, -(0.5 * (NY(i, j - 1, 2) + NY(i, j, 2))) * fE};
      means(uu, vv, ww, mmu);
      visc_normal(val, ax, ay, snx, sny, mmu, uu, vv, ww, fn);
    }
  }

  // spectral radius, Ducros/pressure sensor and dissipation through the face
  // between cells L and R (rhs/spectralradius_i.F, ducrosfordnc_i.F,
  // dissipation_ducros_i.F); ksf: the pressure-sensor field of the face's
  // direction (S_KSI or S_KSJ).
  template <int DIR>
  BCG_HD void dissipation(int iL, int jL, int iR, int jR, int ksf, double fnx, double fny, const S pred[5],
                          S diss[5]) const {
    // Roe average: rr = sqrt(rhoL)/(sqrt(rhoL)+sqrt(rhoR)), so
    // u = (sL uL + sR uR)/(sL + sR), and likewise v and c^2
    const S inv = 1.0 / (P(F_SR, iL, jL) + P(F_SR, iR, jR));
    const S u = (P(F_SU, iL, jL) + P(F_SU, iR, jR)) * inv, v = (P(F_SV, iL, jL) + P(F_SV, iR, jR)) * inv;
    const S c2x = (P(F_SC, iL, jL) + P(F_SC, iR, jR)) * inv;
    const double nx2 = fnx * fnx + fny * fny;
    S un;
    if constexpr (RECT) un = DIR == 1 ? fnx * u : fny * v;
    else un = fnx * u + fny * v;
    const S rspec = fabs_t(un) + sqrt_r(c2x * nx2);
    if (c.k2 == 0.0) {
      // with k2 = 0 the sensor is multiplied by zero (0 * coef = 0 for the
      // finite coef of a physical state, and so is its tangent): eps2 = 0,
      // eps4 = max(0, k4), diss = (rspec eps4) pred
      const S r4 = rspec * (0.0 < c.k4 ? c.k4 : 0.0);
#pragma unroll
      for (int v5 = 0; v5 < 5; ++v5) diss[v5] = r4 * pred[v5];
      return;
    }
    S eps2, eps4;
    {
      // sensor of cells R (1) and L (2): ks and Ducros from pass 2
      const S ks1 = SG(ksf, iR, jR), ks2 = SG(ksf, iL, jL);
      const S ducros1 = SG(S_DUC, iR, jR), ducros2 = SG(S_DUC, iL, jL);
      // dxm = (1 - tanh(arg)) / 2, arg = 2.5 + 10 vol div(u) / (c |n| + 1e-15),
      // decreases with arg: MAX(dxm1, dxm2) is the dxm of the smaller
      // argument.  Arguments closer than rounding could order differently take
      // both tanh and the reference's rule (MAX keeps its first argument unless
      // it is strictly smaller).
      const double nabs = RECT ? (DIR == 1 ? fabs(fnx) : fabs(fny)) : sqrt(nx2);
      const S arg1 = 2.5 + SG(S_ARG, iR, jR) / (SG(S_CS, iR, jR) * nabs + 1e-15);
      const S arg2 = 2.5 + SG(S_ARG, iL, jL) / (SG(S_CS, iL, jL) * nabs + 1e-15);
      const double gap = val(arg1) - val(arg2), tol = 1e-12 * (fabs(val(arg1)) + 1.0);
      S dxm;
      if (gap > tol) {
        dxm = 0.5 * (1.0 - tanh_t(arg2));
      } else if (gap < -tol) {
        dxm = 0.5 * (1.0 - tanh_t(arg1));
      } else {
        dxm = fmax_t(0.5 * (1.0 - tanh_t(arg1)), 0.5 * (1.0 - tanh_t(arg2)));
      }
      const S coef = fmax_t(ks1, ks2) * fmax_t(ducros1, ducros2) * dxm;
      eps2 = c.k2 * coef;
      eps4 = fmax_t(Planes<S>::c(0.0), c.k4 - eps2 * 12.0);
    }
    // rspec (eps2 (wR - wL) / 2 + eps4 pred) with the face factors formed once
    const S re2 = (0.5 * rspec) * eps2, re4 = rspec * eps4;
#pragma unroll
    for (int v5 = 1; v5 <= 5; ++v5) diss[v5 - 1] = re2 * (W(iR, jR, v5) - W(iL, jL, v5)) + re4 * pred[v5 - 1];
  }

  // flux assembly (rhs/fluxnumassembly_i.F): (fv nx/|n| + gv ny/|n|) |n| = fv nx + gv ny
  BCG_HD void assemble(const S fx[5], const S diss[5], const S fn[4], S h[5]) const {
    h[0] = fx[0] - diss[0];
#pragma unroll
    for (int v5 = 2; v5 <= 5; ++v5) h[v5 - 1] = fx[v5 - 1] - diss[v5 - 1] - fn[v5 - 2];
  }

  // Centred face flux of variable v5 along (di, dj) with the weights already
  // multiplied by the face normal (a = cc fnx, b = cc fny), once per face:
  // sum_n a_n (f(+n-1) + f(-n)) + sum_n b_n (g(+n-1) + g(-n))  (rhs/euler_o6_i.F,
  // the o4, o8 and o10 forms for R = 2, 4, 5); DROP 1 leaves out the g half
  // (b = 0), DROP 2 the f half (a = 0).
  template <int DROP>
  BCG_HD S centred(int v5, int i, int j, int di, int dj, const double a[R], const double b[R]) const {
    S fx;
    if constexpr (DROP != 2) {
      fx = a[0] * (Fl(v5, i, j) + Fl(v5, i - di, j - dj));
#pragma unroll
      for (int n = 2; n <= R; ++n)
        fx = fx + a[n - 1] * (Fl(v5, i + (n - 1) * di, j + (n - 1) * dj) + Fl(v5, i - n * di, j - n * dj));
    }
    if constexpr (DROP != 1) {
#pragma unroll
      for (int n = 1; n <= R; ++n) {
        const S t = Gl(v5, i + (n - 1) * di, j + (n - 1) * dj) + Gl(v5, i - n * di, j - n * dj);
        if constexpr (DROP == 2) fx = n == 1 ? b[0] * t : fx + b[n - 1] * t;
        else fx = fx + b[n - 1] * t;
      }
    }
    return fx;
  }
  // Predictor sum_n (-1)^n d_n (w(-n) - w(+n-1)), outermost point first
  // (rhs/predictor_7p_i.F; 5p, 9p, 11p for R = 2, 4, 5)
  BCG_HD S predictor(int v5, int i, int j, int di, int dj) const {
    S p = c.dd[R - 1] * W(i - R * di, j - R * dj, v5);
    if (R & 1) p = -p;
#pragma unroll
    for (int n = R - 1; n >= 1; --n) {
      const S t = c.dd[n - 1] * W(i - n * di, j - n * dj, v5);
      p = (n & 1) ? p - t : p + t;
    }
#pragma unroll
    for (int n = 1; n <= R; ++n) {
      const S t = c.dd[n - 1] * W(i + (n - 1) * di, j + (n - 1) * dj, v5);
      p = (n & 1) ? p + t : p - t;
    }
    return p;
  }

  // i-face (i,j), between cells (i-1,j) and (i,j)
  BCG_HD void iface(int i, int j, S h[5]) const {
    S fx[5], pred[5], diss[5], fn[4];
    const double fnx = NX(i, j, 1), fny = NY(i, j, 1);
    double a[R], b[R];
#pragma unroll
    for (int n = 0; n < R; ++n) { a[n] = c.cc[n] * fnx; b[n] = c.cc[n] * fny; }
#pragma unroll
    for (int v5 = 1; v5 <= 5; ++v5) {
      fx[v5 - 1] = centred<RECT ? 1 : 0>(v5, i, j, 1, 0, a, b);
      pred[v5 - 1] = predictor(v5, i, j, 1, 0);
    }
    visc_i(i, j, ALL_O2 || (c.wall && j <= 2), fnx, fny, fn);
    dissipation<1>(i - 1, j, i, j, S_KSI, fnx, fny, pred, diss);
    assemble(fx, diss, fn, h);
  }

  // j-face (i,j), between cells (i,j-1) and (i,j); j >= 2 with a wall
  BCG_HD void jface(int i, int j, S h[5]) const {
    S fx[5], pred[5], diss[5], fn[4];
    const double fnx = NX(i, j, 2), fny = NY(i, j, 2);
    double a[R], b[R];
#pragma unroll
    for (int n = 0; n < R; ++n) { a[n] = c.cc[n] * fnx; b[n] = c.cc[n] * fny; }
#pragma unroll
    for (int v5 = 1; v5 <= 5; ++v5) {
      if (j > R || !c.wall) {
        fx[v5 - 1] = centred<RECT ? 2 : 0>(v5, i, j, 0, 1, a, b);
      } else {
        // off-centred flux of wall row j from rows 1..NW (rhs/nearbndfluxes5demi_7p.F, 3demi, ...)
        const double* cw = c.cw[j - 2];
        if constexpr (RECT) {
          S sg = cw[0] * Gl(v5, i, 1);
#pragma unroll
          for (int n = 1; n < NW; ++n) sg = sg + cw[n] * Gl(v5, i, n + 1);
          fx[v5 - 1] = sg * fny;
        } else {
          S sf = cw[0] * Fl(v5, i, 1), sg = cw[0] * Gl(v5, i, 1);
#pragma unroll
          for (int n = 1; n < NW; ++n) {
            sf = sf + cw[n] * Fl(v5, i, n + 1);
            sg = sg + cw[n] * Gl(v5, i, n + 1);
          }
          fx[v5 - 1] = sf * fnx + sg * fny;
        }
      }
      pred[v5 - 1] = predictor(v5, i, j, 0, 1);
    }
    visc_j(i, j, ALL_O2 || (c.wall && j == 2), fnx, fny, fn);
    dissipation<2>(i, j - 1, i, j, S_KSJ, fnx, fny, pred, diss);
    assemble(fx, diss, fn, h);
  }

  // adiabatic no-slip wall face j = 1 (rhs/fluxwall.F)
  BCG_HD void wallface(int i, S h[5]) const {
    const int j = 1;
    const S pw = c.ct0 * P(F_P, i, j) + c.ct1 * P(F_P, i, j + 1);
    const S mmu = P(F_MU, i, j);
    const double nx2 = NX(i, j, 2), ny2 = NY(i, j, 2), vf = VOLF(i, j, 2);
    const S ux = 2.0 * P(F_U, i, j) * nx2 * vf, vx = 2.0 * P(F_V, i, j) * nx2 * vf, wx = 2.0 * P(F_W, i, j) * nx2 * vf;
    const S uy = 2.0 * P(F_U, i, j) * ny2 * vf, vy = 2.0 * P(F_V, i, j) * ny2 * vf, wy = 2.0 * P(F_W, i, j) * ny2 * vf;
    const double TWOTHIRD = 2.0 / 3.0;
    const S fvrou = TWOTHIRD * mmu * (2.0 * ux - vy), fvrov = mmu * (uy + vx), fvrow = mmu * (wx);
    const S gvrou = mmu * (uy + vx), gvrov = TWOTHIRD * mmu * (-ux + 2.0 * vy), gvrow = mmu * (wy);
    h[0] = Planes<S>::c(0.0);
    h[1] = pw * nx2 - (fvrou * nx2 + gvrou * ny2);
    h[2] = pw * ny2 - (fvrov * nx2 + gvrov * ny2);
    h[3] = -(fvrow * nx2 + gvrow * ny2);
    h[4] = Planes<S>::c(0.0);
  }
};

// node t of the (im+1) x (jm+1) node set, i fastest: the i-face (j <= jm)
// and the j-face (i <= im) of the node into hn (5 i-face, 5 j-face fields)
template <class S, int R = 3, bool RECT = false>
BCG_HD void face_node(const FaceCtx<S, R, RECT>& fc, const Scratch<S>& hn, int t) {
  const Ext& e = fc.e;
  const int nI = e.im + 1;
  const int i = 1 + t % nI, j = 1 + t / nI;
  S h[5];
  if (j <= e.jm) {
    fc.iface(i, j, h);
#pragma unroll
    for (int v5 = 0; v5 < 5; ++v5) hn.st(v5, t, h[v5]);
  }
  if (i <= e.im) {
    if (j == 1 && fc.c.wall) fc.wallface(i, h); else fc.jface(i, j, h);
#pragma unroll
    for (int v5 = 0; v5 < 5; ++v5) hn.st(5 + v5, t, h[v5]);
  }
}

// balance (rhs/balance.F) of interior cell t: residu = -(h1(i+1)-h1(i)) - (h2(j+1)-h2(j))
template <class S>
BCG_HD void balance_cell(const Ext& e, const Scratch<S>& hn, double* __restrict__ res, double* __restrict__ resd,
                         size_t dstride, int t) {
  const int i = 1 + t % e.im, j = 1 + t / e.im;
  const int nI = e.im + 1;
  const int a = (i - 1) + (j - 1) * nI;
  const size_t q = e.cidx(i, j);
  constexpr int K = NDir<S>::value;
#pragma unroll
  for (int v5 = 0; v5 < 5; ++v5) {
    const S r = -(hn.ld(v5, a + 1) - hn.ld(v5, a)) - (hn.ld(5 + v5, a + nI) - hn.ld(5 + v5, a));
    if constexpr (K == 0) {
      if (res) res[q + (size_t)v5 * e.np] = r;
    } else {
      if (res) res[q + (size_t)v5 * e.np] = r.v;
#pragma unroll
      for (int k = 0; k < K; ++k) resd[(size_t)k * dstride + q + (size_t)v5 * e.np] = r.d[k];
    }
  }
}

}  // namespace bcg
