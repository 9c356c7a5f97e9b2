// Test infrastructure only: CPU oracle for the BROADCAST DNC5 hot path.
//
// A plain restatement of the reference Fortran, templated on the scalar type
// of the state so that one source gives
//   T = double      : the primal routines,
//   T = Dual<N>     : their exact forward derivatives (what Tapenade's
//                     srcfv/tangent/*_d.f90 computes, up to rounding),
//   T = OpCount     : the algorithmic floating-point operation count.
// Arithmetic is written in the same evaluation order as the Fortran text so
// that the double instantiation, compiled without contraction
// (-ffp-contract=off), reproduces the reference bit for bit.
//
// Only tests, the smoke check and the CPU-baseline leg of the benchmark use
// this code.  The shipped library never links it.
//
// Arrays follow the reference's f2py layout: Fortran (column-major) order,
// cell arrays indexed (1-gh:im+gh, 1-gh:jm+gh[, nv]), node/face arrays
// (1-gh:im+gh+1, 1-gh:jm+gh+1[, nv]).
#pragma once
#include <cstddef>
#include <cstring>
#include <algorithm>
#include <vector>
#include <cmath>
#include "dual.hpp"

namespace orc {

// Fortran-indexed view of a column-major array with lower bounds (lo, lo).
template <class T>
struct FArr {
  T* p;
  int ni, nj, lo;
  FArr(T* p_, int ni_, int nj_, int lo_) : p(p_), ni(ni_), nj(nj_), lo(lo_) {}
  inline T& operator()(int i, int j, int v = 1) const {
    return p[(size_t)(i - lo) + (size_t)(j - lo) * ni + (size_t)(v - 1) * ni * nj];
  }
};

struct Consts {
  double cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4;
};

// ===========================================================================
// Stencil coefficients of the DNC schemes of order 3, 5, 7, 9 with R = (order+1)/2
// point pairs (srcfv/rhs/flux_num_dnc{3,5,7,9}.F90 and rhs/coefnearbnd_*.F):
//   bb[0..R-2]  cell-gradient weights        (rhs/gradop_{3,5,7,9}p{i,j}.F)
//   cc[0..R-1]  centred face-flux weights    (rhs/euler_o{4,6,8,10}_{i,j}.F)
//   dd[0..R-1]  predictor weights            (rhs/predictor_{5,7,9,11}p_{i,j}.F)
//   cw[r][0..nw-1]  off-centred j-flux weights of wall row j = r + 2, from the
//               first nw cell rows (rhs/nearbndfluxes{3,5,7,9}demi_*.F)
// Each value is formed by the same floating-point operations as the reference.
// ===========================================================================
struct DncCoefs {
  int order, R, nw;
  double bb[4], cc[5], dd[5], cw[4][11];
};

inline DncCoefs dnc_coefs(int order) {
  DncCoefs k{};
  k.order = order;
  k.R = (order + 1) / 2;
  double denom;
  if (order == 3) {  // flux_num_dnc3.F90:104-123
    denom = 1.0 / 12.0;
    k.bb[0] = 0.5;
    k.cc[0] = 7.0 * denom; k.cc[1] = -denom;
    k.dd[0] = 3.0 * denom; k.dd[1] = denom;
    k.nw = 2;  // face 3/2: c3d0 = c3d1 = 1/2 (:172-173)
    k.cw[0][0] = 0.5; k.cw[0][1] = 0.5;
  } else if (order == 5) {  // flux_num_dnc5.F90:89-118, rhs/coefnearbnd_7p.F with denom 1/60
    denom = 1.0 / 12.0;
    k.bb[0] = 8.0 * denom; k.bb[1] = -denom;
    denom = 1.0 / 60.0;
    k.cc[0] = 37.0 * denom; k.cc[1] = -8.0 * denom; k.cc[2] = denom;
    k.dd[0] = 10.0 * denom; k.dd[1] = 5.0 * denom; k.dd[2] = denom;
    k.nw = 5;
    const double c3[5] = {12.0, 77.0, -43.0, 17.0, -3.0}, c5[5] = {-3.0, 27.0, 47.0, -13.0, 2.0};
    for (int n = 0; n < 5; ++n) { k.cw[0][n] = c3[n] * denom; k.cw[1][n] = c5[n] * denom; }
  } else if (order == 7) {  // flux_num_dnc7.F90:92-128, rhs/coefnearbnd_9p.F with denom 1/840
    denom = 1.0 / 60.0;
    k.bb[0] = 45.0 * denom; k.bb[1] = -9.0 * denom; k.bb[2] = denom;
    denom = 1.0 / 840.0;
    k.cc[0] = 533.0 * denom; k.cc[1] = -139.0 * denom; k.cc[2] = 29.0 * denom; k.cc[3] = -3.0 * denom;
    denom = 1.0 / 280.0;
    k.dd[0] = 35.0 * denom; k.dd[1] = 21.0 * denom; k.dd[2] = 7.0 * denom; k.dd[3] = 1.0 * denom;
    denom = 1.0 / 840.0;
    k.nw = 9;
    const double c3[9] = {92.0, 1547.0, -1861.0, 2171.0, -1917.0, 1191.0, -489.0, 119.0, -13.0};
    const double c5[9] = {-13.0, 209.0, 1079.0, -769.0, 533.0, -279.0, 99.0, -21.0, 2.0};
    const double c7[9] = {2.0, -31.0, 281.0, 911.0, -517.0, 281.0, -111.0, 27.0, -3.0};
    for (int n = 0; n < 9; ++n) { k.cw[0][n] = c3[n] * denom; k.cw[1][n] = c5[n] * denom; k.cw[2][n] = c7[n] * denom; }
  } else if (order == 9) {  // flux_num_dnc9.F90:100-128, rhs/coefnearbnd_11p.F
    denom = 1.0 / 840.0;
    k.bb[0] = 672.0 * denom; k.bb[1] = -168.0 * denom; k.bb[2] = 32.0 * denom; k.bb[3] = -3.0 * denom;
    denom = 1.0 / 2520.0;
    k.cc[0] = 1627.0 * denom; k.cc[1] = -473.0 * denom; k.cc[2] = 127.0 * denom; k.cc[3] = -23.0 * denom;
    k.cc[4] = 2.0 * denom;
    denom = 1.0 / 1260.0;
    k.dd[0] = 126.0 * denom; k.dd[1] = 84.0 * denom; k.dd[2] = 36.0 * denom; k.dd[3] = 9.0 * denom; k.dd[4] = denom;
    k.nw = 11;
    // face 9/2 from the centred weights, then each lower face from the one
    // above: Phi(f - 1) = Phi(f) - sum a_n f_n
    const double a9[11] = {1.0 / 840.0, -(1.0 / 63.0), 3.0 / 28.0, -(4.0 / 7.0), -11.0 / 30.0, 6.0 / 5.0, -0.5,
                           4.0 / 21.0, -(3.0 / 56.0), 1.0 / 105.0, -(1.0 / 1260.0)};
    const double a7[11] = {-(1.0 / 360.0), 1.0 / 24.0, -(3.0 / 8.0), -(319.0 / 420.0), 1.75, -(21.0 / 20.0),
                           7.0 / 12.0, -0.25, 0.075, -(1.0 / 72.0), 1.0 / 840.0};
    const double a5[11] = {1.0 / 90.0, -(2.0 / 9.0), -(341.0 / 280.0), 8.0 / 3.0, -(7.0 / 3.0), 28.0 / 15.0,
                           -(7.0 / 6.0), 8.0 / 15.0, -(1.0 / 6.0), 2.0 / 63.0, -(1.0 / 360.0)};
    const double a3[11] = {-0.1, -(4609.0 / 2520.0), 4.5, -6.0, 7.0, -6.3, 21.0 * 0.2, -2.0, 9.0 / 14.0, -0.125,
                           1.0 / 90.0};
    const double cen[11] = {k.cc[4], k.cc[3], k.cc[2], k.cc[1], k.cc[0], k.cc[0], k.cc[1], k.cc[2], k.cc[3], k.cc[4], 0.0};
    for (int n = 0; n < 11; ++n) {
      k.cw[3][n] = n < 10 ? cen[n] - a9[n] : -a9[n];
      k.cw[2][n] = k.cw[3][n] - a7[n];
      k.cw[1][n] = k.cw[2][n] - a5[n];
      k.cw[0][n] = k.cw[1][n] - a3[n];
    }
  } else {
    k.order = 0;
  }
  return k;
}

// ===========================================================================
// Residual: srcfv/prepro/flux_num_dnc5.f90 (flattened srcfv/rhs/flux_num_dnc5.F90),
// and with order 3, 7 or 9 srcfv/prepro/flux_num_dnc{3,7,9}.f90: the same
// passes with the stencils of DncCoefs, interior j-faces from row R+1,
// off-centred j-fluxes on rows 2..R, 2nd-order viscous fluxes on row 2 (and
// everywhere for DNC3)
// ===========================================================================
template <class T>
struct Dnc5 {
  int im, jm, gh;
  Consts k;
  // coefficients (flux_num_dnc5.f90:69-122, 938-950)
  double HALF = 0.5, ONE = 1.0, ZERO = 0.0, TWO = 2.0, TWOTHIRD = 2.0 / 3.0, FOURTH = 0.25;
  double TWELFTH = 0.25 / 3.0, TWENTYFOURTH = 1.0 / 24.0, ccross, cpprandtl, cvm1, betas;
  DncCoefs sc;
  int R;
  double ct0, ct1;

  FArr<const T> w;
  FArr<const double> nx, ny, vol, volf;
  std::vector<T> velx_, vely_, velz_, tloc_, p_, mu_, f_, g_, gradu_, gradv_, hn_;
  FArr<T> velx, vely, velz, tloc, p, mu, f, g, gradu, gradv;
  int nni, nnj;  // node extents

  Dnc5(const T* w_, const double* nx_, const double* ny_, const double* vol_, const double* volf_,
       int gh_, const Consts& c, int im_, int jm_, int order = 5)
      : im(im_), jm(jm_), gh(gh_), k(c), sc(dnc_coefs(order)), R(sc.R),
        w(w_, im_ + 2 * gh_, jm_ + 2 * gh_, 1 - gh_),
        nx(nx_, im_ + 2 * gh_ + 1, jm_ + 2 * gh_ + 1, 1 - gh_),
        ny(ny_, im_ + 2 * gh_ + 1, jm_ + 2 * gh_ + 1, 1 - gh_),
        vol(vol_, im_ + 2 * gh_, jm_ + 2 * gh_, 1 - gh_),
        volf(volf_, im_ + 2 * gh_, jm_ + 2 * gh_, 1 - gh_),
        velx(nullptr, 0, 0, 0), vely(nullptr, 0, 0, 0), velz(nullptr, 0, 0, 0), tloc(nullptr, 0, 0, 0),
        p(nullptr, 0, 0, 0), mu(nullptr, 0, 0, 0), f(nullptr, 0, 0, 0), g(nullptr, 0, 0, 0),
        gradu(nullptr, 0, 0, 0), gradv(nullptr, 0, 0, 0) {
    const int ni = im + 2 * gh, nj = jm + 2 * gh, lo = 1 - gh;
    nni = ni + 1; nnj = nj + 1;
    const size_t np = (size_t)ni * nj;
    velx_.assign(np, T(0.0)); vely_.assign(np, T(0.0)); velz_.assign(np, T(0.0));
    tloc_.assign(np, T(0.0)); p_.assign(np, T(0.0)); mu_.assign(np, T(0.0));
    f_.assign(np * 5, T(0.0)); g_.assign(np * 5, T(0.0));
    gradu_.assign(np * 2, T(0.0)); gradv_.assign(np * 2, T(0.0));
    hn_.assign((size_t)nni * nnj * 10, T(0.0));
    velx = FArr<T>(velx_.data(), ni, nj, lo); vely = FArr<T>(vely_.data(), ni, nj, lo);
    velz = FArr<T>(velz_.data(), ni, nj, lo); tloc = FArr<T>(tloc_.data(), ni, nj, lo);
    p = FArr<T>(p_.data(), ni, nj, lo); mu = FArr<T>(mu_.data(), ni, nj, lo);
    f = FArr<T>(f_.data(), ni, nj, lo); g = FArr<T>(g_.data(), ni, nj, lo);
    gradu = FArr<T>(gradu_.data(), ni, nj, lo); gradv = FArr<T>(gradv_.data(), ni, nj, lo);
    cpprandtl = k.cp / k.prandtl;
    cvm1 = ONE / k.cv;
    ccross = TWELFTH * 0.0625;
    betas = k.muref * (k.tref + k.cs) / (std::sqrt(k.tref) * k.tref);
    ct0 = 1.125; ct1 = -0.125;
  }

  inline T& hn(int i, int j, int e, int d) {
    return hn_[(size_t)(i - (1 - gh)) + (size_t)(j - (1 - gh)) * nni + (size_t)(e - 1) * nni * nnj +
               (size_t)(d - 1) * nni * nnj * 5];
  }

  // flux_num_dnc5.f90:125-175 (phys/Primitives.F, phys/viscosity.F)
  void primitives() {
#pragma omp parallel for schedule(static)
    for (int j = 1 - gh; j <= jm + gh; ++j)
      for (int i = 1 - gh; i <= im + gh; ++i) {
        const T ro = w(i, j, 1);
        const T rom1 = ONE / ro;
        velx(i, j) = w(i, j, 2) * rom1;
        vely(i, j) = w(i, j, 3) * rom1;
        velz(i, j) = w(i, j, 4) * rom1;
        const T ec = HALF * (velx(i, j) * velx(i, j) + vely(i, j) * vely(i, j) + velz(i, j) * velz(i, j));
        const T eloc = (w(i, j, 5) - ec * ro) * rom1;
        tloc(i, j) = eloc * cvm1;
        p(i, j) = (k.gam - ONE) * ro * eloc;
        const T htot = (w(i, j, 5) + p(i, j)) * rom1;
        f(i, j, 1) = w(i, j, 2);
        f(i, j, 2) = w(i, j, 2) * velx(i, j) + p(i, j);
        f(i, j, 3) = w(i, j, 2) * vely(i, j);
        f(i, j, 4) = w(i, j, 2) * velz(i, j);
        f(i, j, 5) = w(i, j, 2) * htot;
        g(i, j, 1) = w(i, j, 3);
        g(i, j, 2) = w(i, j, 3) * velx(i, j);
        g(i, j, 3) = w(i, j, 3) * vely(i, j) + p(i, j);
        g(i, j, 4) = w(i, j, 3) * velz(i, j);
        g(i, j, 5) = w(i, j, 3) * htot;
        mu(i, j) = betas / (tloc(i, j) + k.s_suth) * sqrt_t(tloc(i, j)) * tloc(i, j);
      }
  }

  // flux_num_dnc5.f90:179-257 (rhs/gradop_5pi.F, gradop_5pj.F, gradient.F,
  // gradveloingh.F).  Only the u and v gradients reach the residual (Ducros
  // sensor); the w and mu gradients of the reference are dead code.
  void gradients() {
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        T gui = sc.bb[0] * (velx(i + 1, j) - velx(i - 1, j)), gvi = sc.bb[0] * (vely(i + 1, j) - vely(i - 1, j));
        T guj = sc.bb[0] * (velx(i, j + 1) - velx(i, j - 1)), gvj = sc.bb[0] * (vely(i, j + 1) - vely(i, j - 1));
        for (int n = 2; n < R; ++n) {
          gui = gui + sc.bb[n - 1] * (velx(i + n, j) - velx(i - n, j));
          gvi = gvi + sc.bb[n - 1] * (vely(i + n, j) - vely(i - n, j));
          guj = guj + sc.bb[n - 1] * (velx(i, j + n) - velx(i, j - n));
          gvj = gvj + sc.bb[n - 1] * (vely(i, j + n) - vely(i, j - n));
        }
        const double volm1 = ONE / vol(i, j);
        const double dxm1 = HALF * (nx(i, j, 1) + nx(i + 1, j, 1)) * volm1;
        const double dxm2 = HALF * (nx(i, j, 2) + nx(i, j + 1, 2)) * volm1;
        const double dym1 = HALF * (ny(i, j, 1) + ny(i + 1, j, 1)) * volm1;
        const double dym2 = HALF * (ny(i, j, 2) + ny(i, j + 1, 2)) * volm1;
        gradu(i, j, 1) = dxm1 * gui + dxm2 * guj;
        gradv(i, j, 1) = dxm1 * gvi + dxm2 * gvj;
        gradu(i, j, 2) = dym1 * gui + dym2 * guj;
        gradv(i, j, 2) = dym1 * gvi + dym2 * gvj;
      }
    // ghost extrapolation, twice, full-range slices as in gradveloingh.F
    const int lo = 1 - gh;
    for (int it = 1; it <= 2; ++it)
      for (int h = 1; h <= gh; ++h) {
        for (int c = 1; c <= 2; ++c)
          for (int i = lo; i <= im + gh; ++i) {
            gradu(i, 1 - h, c) = TWO * gradu(i, 2 - h, c) - gradu(i, 3 - h, c);
          }
        for (int c = 1; c <= 2; ++c)
          for (int i = lo; i <= im + gh; ++i) gradv(i, 1 - h, c) = TWO * gradv(i, 2 - h, c) - gradv(i, 3 - h, c);
        for (int c = 1; c <= 2; ++c)
          for (int i = lo; i <= im + gh; ++i)
            gradu(i, jm + h, c) = TWO * gradu(i, jm - 1 + h, c) - gradu(i, jm - 2 + h, c);
        for (int c = 1; c <= 2; ++c)
          for (int i = lo; i <= im + gh; ++i)
            gradv(i, jm + h, c) = TWO * gradv(i, jm - 1 + h, c) - gradv(i, jm - 2 + h, c);
        for (int c = 1; c <= 2; ++c)
          for (int j = lo; j <= jm + gh; ++j) gradu(1 - h, j, c) = TWO * gradu(2 - h, j, c) - gradu(3 - h, j, c);
        for (int c = 1; c <= 2; ++c)
          for (int j = lo; j <= jm + gh; ++j) gradv(1 - h, j, c) = TWO * gradv(2 - h, j, c) - gradv(3 - h, j, c);
        for (int c = 1; c <= 2; ++c)
          for (int j = lo; j <= jm + gh; ++j)
            gradu(im + h, j, c) = TWO * gradu(im - 1 + h, j, c) - gradu(im - 2 + h, j, c);
        for (int c = 1; c <= 2; ++c)
          for (int j = lo; j <= jm + gh; ++j)
            gradv(im + h, j, c) = TWO * gradv(im - 1 + h, j, c) - gradv(im - 2 + h, j, c);
      }
  }

  // 4-point interpolation row used by the cross terms (rhs/flux_visqueux_o4_i.F)
  static inline T q4(const T& a, const T& b, const T& c, const T& d) { return -a + 9.0 * b + 9.0 * c - d; }

  // --- i-face pieces -------------------------------------------------------
  // Centred face flux (rhs/euler_o6_i.F; o4, o8, o10 for DNC3, 7, 9):
  // (sum_n c_n (f(i+n-1) + f(i-n))) nx + (same for g) ny along direction (di, dj)
  void euler_c(int i, int j, int di, int dj, int dir, T fx[5]) {
    for (int e = 1; e <= 5; ++e) {
      T sf = sc.cc[0] * (f(i, j, e) + f(i - di, j - dj, e));
      T sg = sc.cc[0] * (g(i, j, e) + g(i - di, j - dj, e));
      for (int n = 2; n <= R; ++n) {
        sf = sf + sc.cc[n - 1] * (f(i + (n - 1) * di, j + (n - 1) * dj, e) + f(i - n * di, j - n * dj, e));
        sg = sg + sc.cc[n - 1] * (g(i + (n - 1) * di, j + (n - 1) * dj, e) + g(i - n * di, j - n * dj, e));
      }
      fx[e - 1] = sf * nx(i, j, dir) + sg * ny(i, j, dir);
    }
  }
  void euler_i(int i, int j, T fx[5]) { euler_c(i, j, 1, 0, 1, fx); }
  void euler_j(int i, int j, T fx[5]) { euler_c(i, j, 0, 1, 2, fx); }
  // Off-centred near-wall j-flux of row j from rows 1..nw
  // (rhs/nearbndfluxes5demi_7p.F, nearbndfluxes3demi_7p.F and the 5p, 9p, 11p forms)
  void euler_j_wall(int i, int j, T fx[5]) {
    const double* c = sc.cw[j - 2];
    for (int e = 1; e <= 5; ++e) {
      T sf = c[0] * f(i, 1, e), sg = c[0] * g(i, 1, e);
      for (int n = 1; n < sc.nw; ++n) {
        sf = sf + c[n] * f(i, n + 1, e);
        sg = sg + c[n] * g(i, n + 1, e);
      }
      fx[e - 1] = sf * nx(i, j, 2) + sg * ny(i, j, 2);
    }
  }
  // Predictor (rhs/predictor_7p_i.F, _j.F; 5p, 9p, 11p for DNC3, 7, 9):
  //   sum_n (-1)^n d_n (w(i-n) - w(i+n-1)), outermost point first
  void pred_c(int i, int j, int di, int dj, T pr[5]) {
    for (int e = 1; e <= 5; ++e) {
      T acc = sc.dd[R - 1] * w(i - R * di, j - R * dj, e);
      if (R & 1) acc = -acc;
      for (int n = R - 1; n >= 1; --n) {
        const T t = sc.dd[n - 1] * w(i - n * di, j - n * dj, e);
        acc = (n & 1) ? acc - t : acc + t;
      }
      for (int n = 1; n <= R; ++n) {
        const T t = sc.dd[n - 1] * w(i + (n - 1) * di, j + (n - 1) * dj, e);
        acc = (n & 1) ? acc + t : acc - t;
      }
      pr[e - 1] = acc;
    }
  }
  void pred_i(int i, int j, T pr[5]) { pred_c(i, j, 1, 0, pr); }
  void pred_j(int i, int j, T pr[5]) { pred_c(i, j, 0, 1, pr); }

  // viscous fluxes from the face gradients (rhs/flux_visqueux_o4_i.F:80-103)
  void visc_fluxes(const T& mmu, const T& lambda, const T& uu, const T& vv, const T& ww, const T& ux,
                   const T& uy, const T& vx, const T& vy, const T& wx, const T& wy, const T& tx, const T& ty,
                   T fv[4], T gv[4]) {
    fv[0] = TWOTHIRD * mmu * (TWO * ux - vy);
    fv[1] = mmu * (uy + vx);
    fv[2] = mmu * (wx);
    fv[3] = (lambda * tx + uu * fv[0] + vv * fv[1] + ww * fv[2]);
    gv[0] = mmu * (uy + vx);
    gv[1] = TWOTHIRD * mmu * (-ux + TWO * vy);
    gv[2] = mmu * (wy);
    gv[3] = lambda * ty + uu * gv[0] + vv * gv[1] + ww * gv[2];
  }

  // 4th-order viscous flux through i-face (rhs/flux_visqueux_o4_i.F)
  void visc_i_o4(int i, int j, T fv[4], T gv[4]) {
    const double volm1 = volf(i, j, 1);
    const double nx_N = HALF * (nx(i + 1, j, 1) + nx(i, j, 1));
    const double nx_S = -(HALF * (nx(i - 1, j, 1) + nx(i, j, 1)));
    const double nx_O = HALF * (nx(i - 1, j + 1, 2) + nx(i, j + 1, 2));
    const double nx_E = -(HALF * (nx(i - 1, j, 2) + nx(i, j, 2)));
    const double ny_N = HALF * (ny(i + 1, j, 1) + ny(i, j, 1));
    const double ny_S = -(HALF * (ny(i - 1, j, 1) + ny(i, j, 1)));
    const double ny_O = HALF * (ny(i - 1, j + 1, 2) + ny(i, j + 1, 2));
    const double ny_E = -(HALF * (ny(i - 1, j, 2) + ny(i, j, 2)));
    auto grad = [&](FArr<T>& q, T& gx, T& gy) {
      const T vN = TWENTYFOURTH * (-q(i + 1, j) + 26.0 * q(i, j) - q(i - 1, j));
      const T vS = TWENTYFOURTH * (-q(i, j) + 26.0 * q(i - 1, j) - q(i - 2, j));
      auto row = [&](int jj) { return q4(q(i - 2, jj), q(i - 1, jj), q(i, jj), q(i + 1, jj)); };
      const T vE = ccross * (-row(j - 2) + 7.0 * row(j - 1) + 7.0 * row(j) - row(j + 1));
      const T vO = ccross * (-row(j - 1) + 7.0 * row(j) + 7.0 * row(j + 1) - row(j + 2));
      gx = (vN * nx_N + vS * nx_S + vO * nx_O + vE * nx_E) * volm1;
      gy = (vN * ny_N + vS * ny_S + vO * ny_O + vE * ny_E) * volm1;
    };
    T ux, uy, vx, vy, wx, wy, tx, ty;
    grad(velx, ux, uy); grad(vely, vx, vy); grad(velz, wx, wy); grad(tloc, tx, ty);
    const T uu = 0.0625 * q4(velx(i - 2, j), velx(i - 1, j), velx(i, j), velx(i + 1, j));
    const T vv = 0.0625 * q4(vely(i - 2, j), vely(i - 1, j), vely(i, j), vely(i + 1, j));
    const T ww = 0.0625 * q4(velz(i - 2, j), velz(i - 1, j), velz(i, j), velz(i + 1, j));
    const T mmu = 0.0625 * q4(mu(i - 2, j), mu(i - 1, j), mu(i, j), mu(i + 1, j));
    const T lambda = mmu * cpprandtl;
    visc_fluxes(mmu, lambda, uu, vv, ww, ux, uy, vx, vy, wx, wy, tx, ty, fv, gv);
  }
  // 2nd-order viscous flux through i-face (rhs/flux_visqueux_o2_i.F), rows 1-2
  void visc_i_o2(int i, int j, T fv[4], T gv[4]) {
    const double volm1 = volf(i, j, 1);
    const double nx_N = HALF * (nx(i + 1, j, 1) + nx(i, j, 1));
    const double nx_S = -(HALF * (nx(i - 1, j, 1) + nx(i, j, 1)));
    const double nx_O = HALF * (nx(i - 1, j + 1, 2) + nx(i, j + 1, 2));
    const double nx_E = -(HALF * (nx(i - 1, j, 2) + nx(i, j, 2)));
    const double ny_N = HALF * (ny(i + 1, j, 1) + ny(i, j, 1));
    const double ny_S = -(HALF * (ny(i - 1, j, 1) + ny(i, j, 1)));
    const double ny_O = HALF * (ny(i - 1, j + 1, 2) + ny(i, j + 1, 2));
    const double ny_E = -(HALF * (ny(i - 1, j, 2) + ny(i, j, 2)));
    auto grad = [&](FArr<T>& q, T& gx, T& gy) {
      const T vN = q(i, j);
      const T vS = q(i - 1, j);
      const T vE = FOURTH * (q(i, j) + q(i, j - 1) + q(i - 1, j) + q(i - 1, j - 1));
      const T vO = FOURTH * (q(i, j) + q(i, j + 1) + q(i - 1, j) + q(i - 1, j + 1));
      gx = (vN * nx_N + vS * nx_S + vO * nx_O + vE * nx_E) * volm1;
      gy = (vN * ny_N + vS * ny_S + vO * ny_O + vE * ny_E) * volm1;
    };
    T ux, uy, vx, vy, wx, wy, tx, ty;
    grad(velx, ux, uy); grad(vely, vx, vy); grad(velz, wx, wy); grad(tloc, tx, ty);
    const T uu = HALF * (velx(i, j) + velx(i - 1, j));
    const T vv = HALF * (vely(i, j) + vely(i - 1, j));
    const T ww = HALF * (velz(i, j) + velz(i - 1, j));
    const T mmu = HALF * (mu(i, j) + mu(i - 1, j));
    const T lambda = HALF * (mu(i, j) + mu(i - 1, j)) * cpprandtl;
    visc_fluxes(mmu, lambda, uu, vv, ww, ux, uy, vx, vy, wx, wy, tx, ty, fv, gv);
  }
  // 4th-order viscous flux through j-face (rhs/flux_visqueux_o4_j.F)
  void visc_j_o4(int i, int j, T fv[4], T gv[4]) {
    const double volm1 = volf(i, j, 2);
    const double nx_N = HALF * (nx(i + 1, j - 1, 1) + nx(i + 1, j, 1));
    const double nx_S = -(HALF * (nx(i, j - 1, 1) + nx(i, j, 1)));
    const double nx_O = HALF * (nx(i, j + 1, 2) + nx(i, j, 2));
    const double nx_E = -(HALF * (nx(i, j - 1, 2) + nx(i, j, 2)));
    const double ny_N = HALF * (ny(i + 1, j - 1, 1) + ny(i + 1, j, 1));
    const double ny_S = -(HALF * (ny(i, j - 1, 1) + ny(i, j, 1)));
    const double ny_O = HALF * (ny(i, j + 1, 2) + ny(i, j, 2));
    const double ny_E = -(HALF * (ny(i, j - 1, 2) + ny(i, j, 2)));
    auto grad = [&](FArr<T>& q, T& gx, T& gy) {
      auto col = [&](int ii) { return q4(q(ii, j - 2), q(ii, j - 1), q(ii, j), q(ii, j + 1)); };
      const T vN = ccross * (-col(i - 1) + 7.0 * col(i) + 7.0 * col(i + 1) - col(i + 2));
      const T vS = ccross * (-col(i - 2) + 7.0 * col(i - 1) + 7.0 * col(i) - col(i + 1));
      const T vE = TWENTYFOURTH * (-q(i, j) + 26.0 * q(i, j - 1) - q(i, j - 2));
      const T vO = TWENTYFOURTH * (-q(i, j + 1) + 26.0 * q(i, j) - q(i, j - 1));
      gx = (vN * nx_N + vS * nx_S + vO * nx_O + vE * nx_E) * volm1;
      gy = (vN * ny_N + vS * ny_S + vO * ny_O + vE * ny_E) * volm1;
    };
    T ux, uy, vx, vy, wx, wy, tx, ty;
    grad(velx, ux, uy); grad(vely, vx, vy); grad(velz, wx, wy); grad(tloc, tx, ty);
    const T uu = 0.0625 * q4(velx(i, j - 2), velx(i, j - 1), velx(i, j), velx(i, j + 1));
    const T vv = 0.0625 * q4(vely(i, j - 2), vely(i, j - 1), vely(i, j), vely(i, j + 1));
    const T ww = 0.0625 * q4(velz(i, j - 2), velz(i, j - 1), velz(i, j), velz(i, j + 1));
    const T mmu = 0.0625 * q4(mu(i, j - 2), mu(i, j - 1), mu(i, j), mu(i, j + 1));
    const T lambda = mmu * cpprandtl;
    visc_fluxes(mmu, lambda, uu, vv, ww, ux, uy, vx, vy, wx, wy, tx, ty, fv, gv);
  }
  // 2nd-order viscous flux through j-face (rhs/flux_visqueux_o2_j.F), row 2
  void visc_j_o2(int i, int j, T fv[4], T gv[4]) {
    const double volm1 = volf(i, j, 2);
    const double nx_N = HALF * (nx(i + 1, j - 1, 1) + nx(i + 1, j, 1));
    const double nx_S = -(HALF * (nx(i, j - 1, 1) + nx(i, j, 1)));
    const double nx_O = HALF * (nx(i, j + 1, 2) + nx(i, j, 2));
    const double nx_E = -(HALF * (nx(i, j - 1, 2) + nx(i, j, 2)));
    const double ny_N = HALF * (ny(i + 1, j - 1, 1) + ny(i + 1, j, 1));
    const double ny_S = -(HALF * (ny(i, j - 1, 1) + ny(i, j, 1)));
    const double ny_O = HALF * (ny(i, j + 1, 2) + ny(i, j, 2));
    const double ny_E = -(HALF * (ny(i, j - 1, 2) + ny(i, j, 2)));
    auto grad = [&](FArr<T>& q, T& gx, T& gy) {
      const T vN = FOURTH * (q(i, j) + q(i + 1, j) + q(i, j - 1) + q(i + 1, j - 1));
      const T vS = FOURTH * (q(i, j) + q(i - 1, j) + q(i, j - 1) + q(i - 1, j - 1));
      const T vO = q(i, j);
      const T vE = q(i, j - 1);
      gx = (vN * nx_N + vS * nx_S + vO * nx_O + vE * nx_E) * volm1;
      gy = (vN * ny_N + vS * ny_S + vO * ny_O + vE * ny_E) * volm1;
    };
    T ux, uy, vx, vy, wx, wy, tx, ty;
    grad(velx, ux, uy); grad(vely, vx, vy); grad(velz, wx, wy); grad(tloc, tx, ty);
    const T uu = HALF * (velx(i, j) + velx(i, j - 1));
    const T vv = HALF * (vely(i, j) + vely(i, j - 1));
    const T ww = HALF * (velz(i, j) + velz(i, j - 1));
    const T mmu = HALF * (mu(i, j) + mu(i, j - 1));
    const T lambda = HALF * (mu(i, j) + mu(i, j - 1)) * cpprandtl;
    visc_fluxes(mmu, lambda, uu, vv, ww, ux, uy, vx, vy, wx, wy, tx, ty, fv, gv);
  }

  // Spectral radius, sensor and dissipation through the face between cell L
  // and cell R (rhs/spectralradius_i.F, ducrosfordnc_i.F, dissipation_ducros_i.F).
  void dissipation(int iL, int jL, int iR, int jR, int iLL, int jLL, int iRR, int jRR, double fnx, double fny,
                   const T pr[5], T diss[5]) {
    const T rhomr = w(iR, jR, 1);
    const T ur = w(iR, jR, 2) / rhomr;
    const T vr = w(iR, jR, 3) / rhomr;
    const T c2r = k.gam * k.rgaz * tloc(iR, jR);
    const T rhoml = w(iL, jL, 1);
    const T ul = w(iL, jL, 2) / rhoml;
    const T vl = w(iL, jL, 3) / rhoml;
    const T c2l = k.gam * k.rgaz * tloc(iL, jL);
    const T r = sqrt_t(rhomr / rhoml);
    const T rr = ONE / (ONE + r);
    const T omrr = ONE - rr;
    const T u = ul * rr + ur * omrr;
    const T v = vl * rr + vr * omrr;
    const T c2x = c2l * rr + c2r * omrr;
    const double nx2 = fnx * fnx + fny * fny;
    const T ab = fabs_t(fnx * u + fny * v);
    const T sq = sqrt_t(c2x * nx2);
    const T rspec = ab + sq;
    if (k.k2 == 0.0) {
      // eps2 = k2*coef = 0 and eps4 = max(0, k4) exactly for the finite coef
      // of a physical state, so the sensor does not change the result.
      const T eps4 = fmax_t(T(ZERO), T(k.k4));
      for (int e = 1; e <= 5; ++e) diss[e - 1] = rspec * (eps4 * pr[e - 1]);
      return;
    }
    // pressure sensor on the three-point stencils (L-1, L, R) and (LL, L, R)
    const T ks1 = fabs_t(p(iL, jL) - TWO * p(iR, jR) + p(iRR, jRR)) / fabs_t(p(iL, jL) + TWO * p(iR, jR) + p(iRR, jRR));
    const T ks2 = fabs_t(p(iLL, jLL) - TWO * p(iL, jL) + p(iR, jR)) / fabs_t(p(iLL, jLL) + TWO * p(iL, jL) + p(iR, jR));
    T divu = (gradu(iR, jR, 1) + gradv(iR, jR, 2));
    T divu2 = divu * divu;
    T vort2 = (gradv(iR, jR, 1) - gradu(iR, jR, 2)) * (gradv(iR, jR, 1) - gradu(iR, jR, 2));
    const T ducros1 = divu2 / (divu2 + vort2 + 1e-15);
    const T dxm1 = HALF * (ONE - tanh_t(2.5 + 10.0 * vol(iR, jR) / (sqrt_t(c2r * nx2) + 1e-15) * divu));
    divu = (gradu(iL, jL, 1) + gradv(iL, jL, 2));
    divu2 = divu * divu;
    vort2 = (gradv(iL, jL, 1) - gradu(iL, jL, 2)) * (gradv(iL, jL, 1) - gradu(iL, jL, 2));
    const T ducros2 = divu2 / (divu2 + vort2 + 1e-15);
    const T dxm2 = HALF * (ONE - tanh_t(2.5 + 10.0 * vol(iL, jL) / (sqrt_t(c2l * nx2) + 1e-15) * divu));
    const T coef = fmax_t(ks1, ks2) * fmax_t(ducros1, ducros2) * fmax_t(dxm1, dxm2);
    const T eps2 = k.k2 * coef;
    const T eps4 = fmax_t(T(ZERO), k.k4 - eps2 * 12.0);
    for (int e = 1; e <= 5; ++e) {
      const T diff = HALF * (w(iR, jR, e) - w(iL, jL, e));
      diss[e - 1] = rspec * (eps2 * diff + eps4 * pr[e - 1]);
    }
  }

  // rhs/fluxnumassembly_i.F, fluxnumassembly_j.F
  void assemble(int i, int j, int dir, const T fx[5], const T diss[5], const T fv[4], const T gv[4]) {
    const double sc1 = nx(i, j, dir), sc2 = ny(i, j, dir);
    const double sn = std::sqrt(sc1 * sc1 + sc2 * sc2);
    const double invsn = ONE / sn;
    const double nxloc = sc1 * invsn, nyloc = sc2 * invsn;
    hn(i, j, 1, dir) = fx[0] - diss[0];
    for (int e = 2; e <= 5; ++e)
      hn(i, j, e, dir) = fx[e - 1] - diss[e - 1] - (fv[e - 2] * nxloc + gv[e - 2] * nyloc) * sn;
  }

  // i-face (i,j): between cells (i-1,j) and (i,j)
  void iface(int i, int j, bool o2) {
    T fx[5], pr[5], diss[5], fv[4], gv[4];
    euler_i(i, j, fx);
    pred_i(i, j, pr);
    if (o2) visc_i_o2(i, j, fv, gv); else visc_i_o4(i, j, fv, gv);
    dissipation(i - 1, j, i, j, i - 2, j, i + 1, j, nx(i, j, 1), ny(i, j, 1), pr, diss);
    assemble(i, j, 1, fx, diss, fv, gv);
  }
  // j-face (i,j): between cells (i,j-1) and (i,j); offc: the off-centred
  // near-wall formula of row j.
  void jface(int i, int j, bool offc, bool o2) {
    T fx[5], pr[5], diss[5], fv[4], gv[4];
    if (offc) euler_j_wall(i, j, fx); else euler_j(i, j, fx);
    pred_j(i, j, pr);
    if (o2) visc_j_o2(i, j, fv, gv); else visc_j_o4(i, j, fv, gv);
    dissipation(i, j - 1, i, j, i, j - 2, i, j + 1, nx(i, j, 2), ny(i, j, 2), pr, diss);
    assemble(i, j, 2, fx, diss, fv, gv);
  }
  // adiabatic no-slip wall face j=1 (rhs/fluxwall.F)
  void wallface(int i, int j) {
    const T pw = ct0 * p(i, j) + ct1 * p(i, j + 1);
    const T fxrov2 = pw;
    const T mmu = mu(i, j);
    const double nx2 = nx(i, j, 2), ny2 = ny(i, j, 2), vf = volf(i, j, 2);
    const T ux = TWO * velx(i, j) * nx2 * vf;
    const T vx = TWO * vely(i, j) * nx2 * vf;
    const T wx = TWO * velz(i, j) * nx2 * vf;
    const T uy = TWO * velx(i, j) * ny2 * vf;
    const T vy = TWO * vely(i, j) * ny2 * vf;
    const T wy = TWO * velz(i, j) * ny2 * vf;
    const T fvrou2 = TWOTHIRD * mmu * (TWO * ux - vy);
    const T fvrov2 = mmu * (uy + vx);
    const T fvrow2 = mmu * (wx);
    const T gvrou2 = mmu * (uy + vx);
    const T gvrov2 = TWOTHIRD * mmu * (-ux + TWO * vy);
    const T gvrow2 = mmu * (wy);
    hn(i, j, 1, 2) = T(ZERO);
    hn(i, j, 2, 2) = fxrov2 * nx2 - (fvrou2 * nx2 + gvrou2 * ny2);
    hn(i, j, 3, 2) = fxrov2 * ny2 - (fvrov2 * nx2 + gvrov2 * ny2);
    hn(i, j, 4, 2) = -(fvrow2 * nx2 + gvrow2 * ny2);
    hn(i, j, 5, 2) = T(ZERO);
  }

  // wall = false: flux_num_dnc5_nowall_2d (rhs/flux_num_dnc5_nowall.F90:140), the
  // centred fluxes on every row j = 1..jm+1, no near-wall rows, no wall face
  void run(T* residu_, bool wall = true) {
    primitives();
    gradients();
    const bool all_o2 = (R == 2);  // DNC3: rhs/flux_visqueux_o2.F on every row
#pragma omp parallel for schedule(static)
    for (int j = wall ? R + 1 : 1; j <= jm + 1; ++j)
      for (int i = 1; i <= im + 1; ++i) { iface(i, j, all_o2); jface(i, j, false, all_o2); }
    if (wall) {
      for (int j = R; j >= 2; --j)
        for (int i = 1; i <= im + 1; ++i) { iface(i, j, all_o2 || j == 2); jface(i, j, true, all_o2 || j == 2); }
      for (int i = 1; i <= im + 1; ++i) { iface(i, 1, true); wallface(i, 1); }
    }
    FArr<T> res(residu_, im + 2 * gh, jm + 2 * gh, 1 - gh);
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i)
        for (int e = 1; e <= 5; ++e)
          res(i, j, e) = -(hn(i + 1, j, e, 1) - hn(i, j, e, 1)) - (hn(i, j + 1, e, 2) - hn(i, j, e, 2));
  }
};

template <class T>
void flux_num_dnc5_2d(T* residu, const T* w, const double* nx, const double* ny, const double* vol,
                      const double* volf, int gh, const Consts& c, int im, int jm, bool wall = true, int order = 5) {
  Dnc5<T> s(w, nx, ny, vol, volf, gh, c, im, jm, order);
  s.run(residu, wall);
}

// ===========================================================================
// Boundary conditions (srcfv/borders/*.F90 with init_2d.F)
// interf is the Fortran (2,2) array in column-major order:
//   interf = {imin, imax, jmin, jmax}
// loc is one of "Ilo", "Ihi", "Jlo", "Jhi".
// ===========================================================================
struct Side {
  int kdir = 0, i0 = 0, j0 = 0, high = 0, lmin = 1, lmax = 0, imin, jmin, imax, jmax;
  bool ok = true;
  Side(const char* loc, const int* interf) {
    imin = interf[0]; imax = interf[1]; jmin = interf[2]; jmax = interf[3];
    if (!std::strncmp(loc, "Ilo", 3)) { kdir = 1; i0 = 1; lmax = jmax - jmin + 1; }
    else if (!std::strncmp(loc, "Ihi", 3)) { kdir = 1; i0 = -1; lmax = jmax - jmin + 1; high = 1; }
    else if (!std::strncmp(loc, "Jlo", 3)) { kdir = 2; j0 = 1; lmax = imax - imin + 1; }
    else if (!std::strncmp(loc, "Jhi", 3)) { kdir = 2; j0 = -1; lmax = imax - imin + 1; high = 1; }
    else ok = false;
  }
  int li(int l) const { return imin + (l - lmin) * j0 * j0; }
  int lj(int l) const { return jmin + (l - lmin) * i0 * i0; }
};

// bc_wall_viscous_adia_2d (borders/bc_wall_viscous.F90:2-99)
template <class T>
void bc_wall_viscous_adia_2d(T* w_, const char* loc, double gam, const int* interf, int gh, int im, int jm) {
  FArr<T> w(w_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  Side s(loc, interf);
  const double gam1 = gam - 1.0, gami = 1.0 / gam, ct0 = 1.125, ct1 = -0.125, THIRD = 1.0 / 3.0, FOUR = 4.0,
               HALF = 0.5, ONE = 1.0;
  const int i0 = s.i0, j0 = s.j0;
  for (int l = s.lmin; l <= s.lmax; ++l) {
    const int i = s.li(l), j = s.lj(l);
    const T roe = w(i, j, 1);
    T roem1 = ONE / roe;
    const T ue = w(i, j, 2) * roem1, ve = w(i, j, 3) * roem1, we = w(i, j, 4) * roem1;
    const T ve2 = ue * ue + ve * ve;
    const T pe = gam1 * (w(i, j, 5) - HALF * roe * ve2);
    const T roe1 = w(i + i0, j + j0, 1);
    const T roe1m1 = ONE / roe1;
    const T ue1 = w(i + i0, j + j0, 2) * roe1m1, ve1 = w(i + i0, j + j0, 3) * roe1m1;
    const T ve21 = ue1 * ue1 + ve1 * ve1;
    const T pe1 = gam1 * (w(i + i0, j + j0, 5) - HALF * roe1 * ve21);
    const T pw = ct0 * pe + ct1 * pe1;
    const T pi = THIRD * (FOUR * pw - pe);
    T roi = pow_t(pi / pe * pow_t(roe, gam), gami);
    T ui = -ue, vi = -ve, wi = -we;
    T roiei = pi / gam1 + HALF * roi * (ui * ui + vi * vi);
    for (int de = 1; de <= gh; ++de) {
      w(i - de * i0, j - de * j0, 1) = roi;
      w(i - de * i0, j - de * j0, 2) = roi * ui;
      w(i - de * i0, j - de * j0, 3) = roi * vi;
      w(i - de * i0, j - de * j0, 4) = roi * wi;
      w(i - de * i0, j - de * j0, 5) = roiei;
      roi = w(i + de * i0, j + de * j0, 1);
      roem1 = ONE / roi;
      const T a = w(i + de * i0, j + de * j0, 2) * roem1;
      const T b = w(i + de * i0, j + de * j0, 3) * roem1;
      const T c = w(i + de * i0, j + de * j0, 4) * roem1;
      roiei = w(i + de * i0, j + de * j0, 5);
      ui = -a; vi = -b; wi = -c;
    }
  }
}

// bc_no_reflexion_2d (borders/bc_no_reflexion.F90:8-152); wbd is (lm,5)
template <class T>
void bc_no_reflexion_2d(T* w_, const double* wbd_, int lm, const char* loc, const int* interf, const double* nx_,
                        const double* ny_, double gam, int gh, int im, int jm) {
  FArr<T> w(w_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  FArr<const double> nx(nx_, im + 2 * gh + 1, jm + 2 * gh + 1, 1 - gh), ny(ny_, im + 2 * gh + 1, jm + 2 * gh + 1, 1 - gh);
  auto wbd = [&](int l, int v) { return wbd_[(size_t)(l - 1) + (size_t)(v - 1) * lm]; };
  Side s(loc, interf);
  const double ONE = 1.0, HALF = 0.5, TWO = 2.0, gam1 = gam - ONE;
  const double sens = (double)(s.i0 + s.j0);
  const int i1 = s.i0 * s.i0, j1 = s.j0 * s.j0, i0 = s.i0, j0 = s.j0;
  for (int l = s.lmin; l <= s.lmax; ++l) {
    const int i = s.imin + (l - s.lmin) * j1, j = s.jmin + (l - s.lmin) * i1;
    const double nxloc = nx(i + s.high * i1, j + s.high * j1, s.kdir);
    const double nyloc = ny(i + s.high * i1, j + s.high * j1, s.kdir);
    const double nsum = std::sqrt(nxloc * nxloc + nyloc * nyloc);
    const double nsumi = ONE / nsum;
    const double nxnorm = nxloc * nsumi * sens, nynorm = nyloc * nsumi * sens;
    const T ro0 = w(i, j, 1);
    const T ro0m1 = ONE / ro0;
    const T uu = w(i, j, 2) * ro0m1, vv = w(i, j, 3) * ro0m1, ww = w(i, j, 4) * ro0m1;
    const T roe1 = w(i, j, 5) - HALF * ro0 * (uu * uu + vv * vv + ww * ww);
    const T p0 = gam1 * (roe1);
    const T roc0 = ro0 * sqrt_t(gam * p0 * ro0m1);
    const T roc0m1 = ONE / roc0;
    const T rovn0 = (w(i, j, 2) * nxnorm + w(i, j, 3) * nynorm);
    const double epsm = HALF + fsign(HALF, roc0 - rovn0);
    const double eps0 = HALF + fsign(HALF, -rovn0);
    const double epsp = HALF + fsign(HALF, -roc0 - rovn0);
    const double rod = wbd(l, 1);
    const double rodm1 = ONE / rod;
    const double ud = wbd(l, 2) * rodm1, vd = wbd(l, 3) * rodm1, wdi = wbd(l, 4) * rodm1;
    const double pd = gam1 * (wbd(l, 5) - rod * HALF * (ud * ud + vd * vd + wdi * wdi));
    const double vnd = (ud * nxnorm + vd * nynorm);
    const double utd = ud - vnd * nxnorm, vtd = vd - vnd * nynorm;
    const T ros = w(i, j, 1);
    const T rosm1 = ONE / ros;
    const T us = w(i, j, 2) * rosm1, vs = w(i, j, 3) * rosm1, ws = w(i, j, 4) * rosm1;
    const T ps = gam1 * (w(i, j, 5) - ros * HALF * (us * us + vs * vs + ws * ws));
    const T vns = (us * nxnorm + vs * nynorm);
    const T uts = us - vns * nxnorm, vts = vs - vns * nynorm;
    const T ut = eps0 * uts + (ONE - eps0) * utd;
    const T vt = eps0 * vts + (ONE - eps0) * vtd;
    const T wt = eps0 * ws + (ONE - eps0) * wdi;
    const T am = epsm * (ps - roc0 * vns) + (ONE - epsm) * (pd - roc0 * vnd);
    const T ap = epsp * (ps + roc0 * vns) + (ONE - epsp) * (pd + roc0 * vnd);
    const T vn = (ap - am) * HALF * roc0m1;
    const T pp = (ap + am) * HALF;
    const T bs = (pp - ps) * ro0 * ro0 * roc0m1 * roc0m1 + ros;
    const T b0 = (pp - pd) * ro0 * ro0 * roc0m1 * roc0m1 + rod;
    T ro = eps0 * bs + (ONE - eps0) * b0;
    const T rom1 = ONE / ro;
    const T roe = pp / gam1;
    T rou = ro * (ut + vn * nxnorm);
    T rov = ro * (vt + vn * nynorm);
    T row = ro * wt;
    T roe2 = roe + HALF * rom1 * (rou * rou + rov * rov + row * row);
    for (int de = 1; de <= gh; ++de) {
      const int da = de - 1;
      w(i - de * i0, j - de * j0, 1) = ro;
      w(i - de * i0, j - de * j0, 2) = rou;
      w(i - de * i0, j - de * j0, 3) = rov;
      w(i - de * i0, j - de * j0, 4) = row;
      w(i - de * i0, j - de * j0, 5) = roe2;
      ro = TWO * ro - w(i - da * i0, j - da * j0, 1);
      rou = TWO * rou - w(i - da * i0, j - da * j0, 2);
      rov = TWO * rov - w(i - da * i0, j - da * j0, 3);
      row = TWO * row - w(i - da * i0, j - da * j0, 4);
      roe2 = TWO * roe2 - w(i - da * i0, j - da * j0, 5);
    }
  }
}

// bc_supandsubinlet_2d (borders/bc_supandsubinlet.F90:2-171); field is (lm,gh,5)
template <class T>
void bc_supandsubinlet_2d(T* w_, const char* loc, const int* interf, const double* field_, int lm,
                          const double* nx_, const double* ny_, double gam, int im, int jm, int gh) {
  FArr<T> w(w_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  FArr<const double> nx(nx_, im + 2 * gh + 1, jm + 2 * gh + 1, 1 - gh), ny(ny_, im + 2 * gh + 1, jm + 2 * gh + 1, 1 - gh);
  auto field = [&](int a, int b, int v) { return field_[(size_t)(a - 1) + (size_t)(b - 1) * lm + (size_t)(v - 1) * lm * gh]; };
  Side s(loc, interf);
  const double HALF = 0.5, ONE = 1.0, gam1 = gam - ONE;
  const int i0 = s.i0, j0 = s.j0;
  for (int l = s.lmin; l <= s.lmax; ++l) {
    const int i = s.li(l), j = s.lj(l);
    const T wr1 = w(i, j, 1);
    T rom1 = ONE / wr1;
    const T wr2 = w(i, j, 2) * rom1, wr3 = w(i, j, 3) * rom1, wr4 = w(i, j, 4) * rom1;
    const T pr = gam1 * (w(i, j, 5) - wr1 * (wr2 * wr2 + wr3 * wr3 + wr4 * wr4));
    T hr = (w(i, j, 5) + pr) * rom1;
    const double wl1 = field(j, i, 1);
    const double rosm1_ = ONE / wl1;
    const double wl2 = field(j, i, 2) * rosm1_, wl3 = field(j, i, 3) * rosm1_, wl4 = field(j, i, 4) * rosm1_;
    const double pl = gam1 * (field(j, i, 5) - wl1 * (wl2 * wl2 + wl3 * wl3 + wl4 * wl4));
    T hl = T((field(j, i, 5) + pl) * rosm1_);
    T r = sqrt_t(wr1 / wl1);
    T rr = sqrt_t(wr1 * wl1);
    T oneonrplusone = ONE / (r + ONE);
    T uu = (wr2 * r + wl2) * oneonrplusone;
    T vv = (wr3 * r + wl3) * oneonrplusone;
    T ww = (wr4 * r + wl4) * oneonrplusone;
    T hh = (hr * r + hl) * oneonrplusone;
    const T velo2 = uu * uu + vv * vv + ww;
    T ee = HALF * velo2;
    T sound2 = gam1 * (hh - ee);
    const T mach = sqrt_t(velo2 / sound2);
    const bool sub = (mach < ONE);
    double nxnorm = 0.0, nynorm = 0.0, epsm = 0.0, eps0 = 0.0, epsp = 0.0;
    if (sub) {
      const double nxloc = nx(i, j, s.kdir), nyloc = ny(i, j, s.kdir);
      const double nsum = ONE / std::sqrt(nxloc * nxloc + nyloc * nyloc);
      nxnorm = nxloc * nsum; nynorm = nyloc * nsum;
      const T roc0 = rr * sqrt_t(sound2);
      const T rovn0 = rr * (uu * nxnorm + vv * nynorm);
      epsm = HALF + fsign(HALF, roc0 - rovn0);
      eps0 = HALF + fsign(HALF, -rovn0);
      epsp = HALF + fsign(HALF, -roc0 - rovn0);
    }
    for (int de = 1; de <= gh; ++de) {
      for (int v = 1; v <= 5; ++v) w(i - de * i0, j - de * j0, v) = T(field(l, de, v));
      const int da = de - 1;
      if (sub) {
        const T rod = w(i - de * i0, j - de * j0, 1);
        rom1 = ONE / rod;
        const T ud = w(i - de * i0, j - de * j0, 2) * rom1;
        const T vd = w(i - de * i0, j - de * j0, 3) * rom1;
        const T wd = w(i - de * i0, j - de * j0, 4) * rom1;
        const T pd = gam1 * (w(i - de * i0, j - de * j0, 5) - rod * HALF * (ud * ud + vd * vd + wd * wd));
        const T vnd = (ud * nxnorm + vd * nynorm);
        const T utd = ud - vnd * nxnorm, vtd = vd - vnd * nynorm;
        hl = (w(i - de * i0, j - de * j0, 5) + pd) * rom1;
        const T ros = w(i - da * i0, j - da * j0, 1);
        const T rosm1 = ONE / ros;
        const T us = w(i - da * i0, j - da * j0, 2) * rosm1;
        const T vs = w(i - da * i0, j - da * j0, 3) * rosm1;
        const T ws = w(i - da * i0, j - da * j0, 4) * rosm1;
        const T ps = gam1 * (w(i - da * i0, j - da * j0, 5) - ros * HALF * (us * us + vs * vs + ws * ws));
        const T vns = (us * nxnorm + vs * nynorm);
        const T uts = us - vns * nxnorm, vts = vs - vns * nynorm;
        hr = (w(i - da * i0, j - da * j0, 5) + ps) * rosm1;
        r = sqrt_t(ros * rom1);
        rr = sqrt_t(ros * rod);
        oneonrplusone = ONE / (r + ONE);
        uu = (us * r + ud) * oneonrplusone;
        vv = (vs * r + vd) * oneonrplusone;
        ww = (ws * r + wd) * oneonrplusone;
        ee = HALF * (uu * uu + vv * vv + ww * ww);
        hh = (hr * r + hl) * oneonrplusone;
        sound2 = gam1 * (hh - ee);
        const T roc0 = rr * sqrt_t(sound2);
        const T roc0m1 = ONE / roc0;
        const T ut = eps0 * uts + (ONE - eps0) * utd;
        const T vt = eps0 * vts + (ONE - eps0) * vtd;
        const T am = epsm * (ps - roc0 * vns) + (ONE - epsm) * (pd - roc0 * vnd);
        const T ap = epsp * (ps + roc0 * vns) + (ONE - epsp) * (pd + roc0 * vnd);
        const T vn = (ap - am) * HALF * roc0m1;
        const T pp = (ap + am) * HALF;
        const T bs = (pp - ps) * rr * rr * roc0m1 * roc0m1 + ros;
        const T b0 = (pp - pd) * rr * rr * roc0m1 * roc0m1 + rod;
        const T ro = eps0 * bs + (ONE - eps0) * b0;
        const T roe = pp / gam1;
        const T rou = ro * (ut + vn * nxnorm);
        const T rov = ro * (vt + vn * nynorm);
        const T row = T(field(j, de, 4));
        w(i - de * i0, j - de * j0, 1) = ro;
        w(i - de * i0, j - de * j0, 2) = rou;
        w(i - de * i0, j - de * j0, 3) = rov;
        w(i - de * i0, j - de * j0, 4) = row;
        w(i - de * i0, j - de * j0, 5) = roe + HALF * (rou * rou + rov * rov + row * row) / ro;
      }
    }
  }
}

// bc_extrapolate_o2_2d (borders/bc_extrapolate.F90:39-71)
template <class T>
void bc_extrapolate_o2_2d(T* w_, const char* loc, const int* interf, int im, int jm, int gh, int em) {
  FArr<T> w(w_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  Side s(loc, interf);
  const int i0 = s.i0, j0 = s.j0;
  for (int l = s.lmin; l <= s.lmax; ++l) {
    const int i = s.li(l), j = s.lj(l);
    for (int de = 1; de <= gh; ++de) {
      const int e1 = de - 1, e2 = de - 2;
      for (int v = 1; v <= em; ++v)
        w(i - i0 * de, j - j0 * de, v) = 2.0 * w(i - i0 * e1, j - j0 * e1, v) - w(i - i0 * e2, j - j0 * e2, v);
    }
  }
}

// jn_match_2d (borders/jn_match.F90:3-66): copy of a block of cells.  Arrays
// are (1-gh1:im+gh2, 1-gh3:jm+gh4, em); prr/prd are Fortran (2,2) column-major
// {imin, imax, jmin, jmax}; tr is (2).
template <class T>
void jn_match_2d(T* wr_, const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr, int jmr, const T* wd_,
                 const int* prd, int gh1d, int gh2d, int gh3d, int gh4d, int imd, int jmd, const int* tr, int em) {
  const int nir = imr + gh1r + gh2r, njr = jmr + gh3r + gh4r;
  const int nid = imd + gh1d + gh2d, njd = jmd + gh3d + gh4d;
  auto WR = [&](int i, int j, int v) -> T& { return wr_[(size_t)(i - (1 - gh1r)) + (size_t)(j - (1 - gh3r)) * nir + (size_t)(v - 1) * nir * njr]; };
  auto WD = [&](int i, int j, int v) -> const T& { return wd_[(size_t)(i - (1 - gh1d)) + (size_t)(j - (1 - gh3d)) * nid + (size_t)(v - 1) * nid * njd]; };
  auto P = [](const int* a, int r, int c) { return a[(r - 1) + (c - 1) * 2]; };
  const int istep = tr[0] >= 0 ? 1 : -1, jstep = tr[1] >= 0 ? 1 : -1;
  const int idir = std::abs(tr[0]), jdir = std::abs(tr[1]);
  int i1, i2, j1, j2;
  if (istep == 1) { i1 = 1; i2 = P(prd, 2, idir) - P(prd, 1, idir) + 1; } else { i1 = P(prd, 2, idir) - P(prd, 1, idir) + 1; i2 = 1; }
  if (jstep == 1) { j1 = 1; j2 = P(prd, 2, jdir) - P(prd, 1, jdir) + 1; } else { j1 = P(prd, 2, jdir) - P(prd, 1, jdir) + 1; j2 = 1; }
  int idd = 1, jdd = 1;
  for (int j = j1; jstep > 0 ? j <= j2 : j >= j2; j += jstep) {
    for (int i = i1; istep > 0 ? i <= i2 : i >= i2; i += istep) {
      const int ir = P(prr, 1, 1) + idd - 1, jr = P(prr, 1, 2) + jdd - 1;
      const int id = P(prd, 1, idir) + i - 1, jd = P(prd, 1, jdir) + j - 1;
      for (int v = 1; v <= em; ++v) WR(ir, jr, v) = WD(id, jd, v);
      ++idd;
    }
    idd = 1; ++jdd;
  }
}

// ===========================================================================
// Geometry (srcfv/prepro/computegeom.f90), double only
// ===========================================================================
inline void computegeom_2d(double* x0_, double* y0_, double* nx_, double* ny_, double* xc_, double* yc_,
                           double* vol_, double* volf_, int im, int jm, int gh) {
  const int lo = 1 - gh, nni = im + 2 * gh + 1, nnj = jm + 2 * gh + 1, ni = im + 2 * gh, nj = jm + 2 * gh;
  FArr<double> x0(x0_, nni, nnj, lo), y0(y0_, nni, nnj, lo), nx(nx_, nni, nnj, lo), ny(ny_, nni, nnj, lo);
  FArr<double> xc(xc_, ni, nj, lo), yc(yc_, ni, nj, lo), vol(vol_, ni, nj, lo), volf(volf_, ni, nj, lo);
  const double TWO = 2.0, HALF = 0.5, FOURTH = 0.25;
  for (int g = 1; g <= gh; ++g)
    for (int dummy = 1; dummy <= 2; ++dummy) {
      for (int j = lo; j <= jm + gh + 1; ++j) x0(1 - g, j) = TWO * x0(2 - g, j) - x0(3 - g, j);
      for (int j = lo; j <= jm + gh + 1; ++j) x0(im + 1 + g, j) = TWO * x0(im + g, j) - x0(im - 1 + g, j);
      for (int i = lo; i <= im + gh + 1; ++i) x0(i, 1 - g) = TWO * x0(i, 2 - g) - x0(i, 3 - g);
      for (int i = lo; i <= im + gh + 1; ++i) x0(i, jm + 1 + g) = TWO * x0(i, jm + g) - x0(i, jm - 1 + g);
      for (int i = lo; i <= im + gh + 1; ++i) y0(i, 1 - g) = TWO * y0(i, 2 - g) - y0(i, 3 - g);
      for (int i = lo; i <= im + gh + 1; ++i) y0(i, jm + 1 + g) = TWO * y0(i, jm + g) - y0(i, jm - 1 + g);
      for (int j = lo; j <= jm + gh + 1; ++j) y0(1 - g, j) = TWO * y0(2 - g, j) - y0(3 - g, j);
      for (int j = lo; j <= jm + gh + 1; ++j) y0(im + 1 + g, j) = TWO * y0(im + g, j) - y0(im - 1 + g, j);
    }
  for (int j = 1; j <= jm + 1; ++j)
    for (int i = 1; i <= im + 1; ++i) {
      xc(i, j) = FOURTH * (x0(i, j) + x0(i + 1, j) + x0(i, j + 1) + x0(i + 1, j + 1));
      yc(i, j) = FOURTH * (y0(i, j) + y0(i + 1, j) + y0(i, j + 1) + y0(i + 1, j + 1));
      const double xa = x0(i, j), ya = y0(i, j), xb = x0(i + 1, j), yb = y0(i + 1, j);
      const double xc1 = x0(i, j + 1), yc1 = y0(i, j + 1), xd = x0(i + 1, j + 1), yd = y0(i + 1, j + 1);
      const double abx = xb - xa, aby = yb - ya, acx = xc1 - xa, acy = yc1 - ya;
      const double q1 = HALF * std::fabs(abx * acy - acx * aby);
      const double dcx = xc1 - xd, dcy = yc1 - yd, dbx = xb - xd, dby = yb - yd;
      const double q2 = HALF * std::fabs(dcx * dby - dbx * dcy);
      vol(i, j) = q1 + q2;
      nx(i, j, 1) = y0(i, j + 1) - y0(i, j);
      ny(i, j, 1) = x0(i, j) - x0(i, j + 1);
      nx(i, j, 2) = y0(i, j) - y0(i + 1, j);
      ny(i, j, 2) = x0(i + 1, j) - x0(i, j);
    }
  for (int g = 1; g <= gh; ++g)
    for (int dummy = 1; dummy <= 2; ++dummy) {
      for (int j = lo; j <= jm + gh; ++j) xc(1 - g, j) = TWO * xc(2 - g, j) - xc(3 - g, j);
      for (int j = lo; j <= jm + gh; ++j) xc(im + g, j) = TWO * xc(im - 1 + g, j) - xc(im - 2 + g, j);
      for (int i = lo; i <= im + gh; ++i) xc(i, 1 - g) = TWO * xc(i, 2 - g) - xc(i, 3 - g);
      for (int i = lo; i <= im + gh; ++i) xc(i, jm + g) = TWO * xc(i, jm - 1 + g) - xc(i, jm - 2 + g);
      for (int j = lo; j <= jm + gh; ++j) yc(1 - g, j) = TWO * yc(2 - g, j) - yc(3 - g, j);
      for (int j = lo; j <= jm + gh; ++j) yc(im + g, j) = TWO * yc(im - 1 + g, j) - yc(im - 2 + g, j);
      for (int i = lo; i <= im + gh; ++i) yc(i, 1 - g) = TWO * yc(i, 2 - g) - yc(i, 3 - g);
      for (int i = lo; i <= im + gh; ++i) yc(i, jm + g) = TWO * yc(i, jm - 1 + g) - yc(i, jm - 2 + g);
      for (int j = 1; j <= jm; ++j) vol(1 - g, j) = TWO * vol(2 - g, j) - vol(3 - g, j);
      for (int j = 1; j <= jm; ++j) vol(im + g, j) = TWO * vol(im - 1 + g, j) - vol(im - 2 + g, j);
      for (int i = lo; i <= im + gh; ++i) vol(i, 1 - g) = TWO * vol(i, 2 - g) - vol(i, 3 - g);
      for (int i = lo; i <= im + gh; ++i) vol(i, jm + g) = TWO * vol(i, jm - 1 + g) - vol(i, jm - 2 + g);
      for (int c = 1; c <= 2; ++c)
        for (int j = lo; j <= jm + gh + 1; ++j) nx(1 - g, j, c) = TWO * nx(2 - g, j, c) - nx(3 - g, j, c);
      for (int c = 1; c <= 2; ++c)
        for (int j = lo; j <= jm + gh + 1; ++j) ny(1 - g, j, c) = TWO * ny(2 - g, j, c) - ny(3 - g, j, c);
      for (int c = 1; c <= 2; ++c)
        for (int j = lo; j <= jm + gh + 1; ++j) nx(im + 1 + g, j, c) = TWO * nx(im + g, j, c) - nx(im - 1 + g, j, c);
      for (int c = 1; c <= 2; ++c)
        for (int j = lo; j <= jm + gh + 1; ++j) ny(im + 1 + g, j, c) = TWO * ny(im + g, j, c) - ny(im - 1 + g, j, c);
      for (int c = 1; c <= 2; ++c)
        for (int i = lo; i <= im + gh + 1; ++i) nx(i, 1 - g, c) = TWO * nx(i, 2 - g, c) - nx(i, 3 - g, c);
      for (int c = 1; c <= 2; ++c)
        for (int i = lo; i <= im + gh + 1; ++i) ny(i, 1 - g, c) = TWO * ny(i, 2 - g, c) - ny(i, 3 - g, c);
      for (int c = 1; c <= 2; ++c)
        for (int i = lo; i <= im + gh + 1; ++i) nx(i, 1 + jm + g, c) = TWO * nx(i, jm + g, c) - nx(i, g + jm - 1, c);
      for (int c = 1; c <= 2; ++c)
        for (int i = lo; i <= im + gh + 1; ++i) ny(i, 1 + jm + g, c) = TWO * ny(i, jm + g, c) - ny(i, g + jm - 1, c);
    }
  for (int j = 1; j <= jm + 1; ++j)
    for (int i = 1; i <= im + 1; ++i) {
      volf(i, j, 1) = TWO / (vol(i, j) + vol(i - 1, j));
      volf(i, j, 2) = TWO / (vol(i, j) + vol(i, j - 1));
    }
}

// ===========================================================================
// Spanwise operators (srcfv/dz)
// ===========================================================================
// Both operators are  out(i,j,e) = sum_k coeffs(i,j,e,k) * d func_k(i,j,e)/dw . wd
// over the interior: the coefficients come from the base flow w, the func_k
// are auxiliary fields of w whose tangents along wd the reference takes from
// Tapenade (dz/function_5p_dz_d.f90, dz/function_5p_dz2_d.f90).  Here the
// func_k are evaluated on Dual<N> numbers.
//
// Cell fields shared by both: rhs/primvisc.F (primitives and Sutherland
// viscosity on every padded cell) and rhs/gradop_5pi.F, gradop_5pj.F,
// geom/dxdy.F, gradient.F (4th-order gradients of u, v, w, mu).
template <class T>
struct SpanFields {
  int im, jm, gh, ni, nj;
  std::vector<T> velx, vely, velz, tloc, p, mu;
  std::vector<T> gu, gv, gw, gmu;  // (x, y) pairs per cell, interior filled
  size_t c(int i, int j) const { return (size_t)(i - (1 - gh)) + (size_t)(j - (1 - gh)) * ni; }

  SpanFields(const T* w_, const double* nx_, const double* ny_, const double* vol_, int gh_, const Consts& k,
             int im_, int jm_, bool gradients)
      : im(im_), jm(jm_), gh(gh_), ni(im_ + 2 * gh_), nj(jm_ + 2 * gh_) {
    const size_t np = (size_t)ni * nj;
    FArr<const T> w(w_, ni, nj, 1 - gh);
    FArr<const double> nx(nx_, ni + 1, nj + 1, 1 - gh), ny(ny_, ni + 1, nj + 1, 1 - gh), vol(vol_, ni, nj, 1 - gh);
    velx.assign(np, T(0.0)); vely.assign(np, T(0.0)); velz.assign(np, T(0.0));
    tloc.assign(np, T(0.0)); p.assign(np, T(0.0)); mu.assign(np, T(0.0));
    const double ONE = 1.0, HALF = 0.5;
    const double cvm1 = ONE / k.cv;
    const double betas = k.muref * (k.tref + k.cs) / (std::sqrt(k.tref) * k.tref);
    for (int j = 1 - gh; j <= jm + gh; ++j)
      for (int i = 1 - gh; i <= im + gh; ++i) {
        const size_t q = c(i, j);
        const T ro = w(i, j, 1);
        const T rom1 = ONE / ro;
        velx[q] = w(i, j, 2) * rom1;
        vely[q] = w(i, j, 3) * rom1;
        velz[q] = w(i, j, 4) * rom1;
        const T ec = HALF * (velx[q] * velx[q] + vely[q] * vely[q] + velz[q] * velz[q]);
        const T eloc = (w(i, j, 5) - ec * ro) * rom1;
        tloc[q] = eloc * cvm1;
        p[q] = (k.gam - ONE) * ro * eloc;
        mu[q] = betas / (tloc[q] + k.s_suth) * sqrt_t(tloc[q]) * tloc[q];
      }
    if (!gradients) return;
    gu.assign(2 * np, T(0.0)); gv.assign(2 * np, T(0.0)); gw.assign(2 * np, T(0.0)); gmu.assign(2 * np, T(0.0));
    const double b1 = 8.0 * (1.0 / 12.0), b2 = -(1.0 / 12.0);
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        auto di = [&](const std::vector<T>& f) {
          return b1 * (f[c(i + 1, j)] - f[c(i - 1, j)]) + b2 * (f[c(i + 2, j)] - f[c(i - 2, j)]);
        };
        auto dj = [&](const std::vector<T>& f) {
          return b1 * (f[c(i, j + 1)] - f[c(i, j - 1)]) + b2 * (f[c(i, j + 2)] - f[c(i, j - 2)]);
        };
        const T gui = di(velx), gvi = di(vely), gwi = di(velz), gmui = di(mu);
        const T guj = dj(velx), gvj = dj(vely), gwj = dj(velz), gmuj = dj(mu);
        const double volm1 = ONE / vol(i, j);
        const double dxm1 = HALF * (nx(i, j, 1) + nx(i + 1, j, 1)) * volm1;
        const double dxm2 = HALF * (nx(i, j, 2) + nx(i, j + 1, 2)) * volm1;
        const double dym1 = HALF * (ny(i, j, 1) + ny(i + 1, j, 1)) * volm1;
        const double dym2 = HALF * (ny(i, j, 2) + ny(i, j + 1, 2)) * volm1;
        const size_t q = 2 * c(i, j);
        gu[q] = dxm1 * gui + dxm2 * guj;   gu[q + 1] = dym1 * gui + dym2 * guj;
        gv[q] = dxm1 * gvi + dxm2 * gvj;   gv[q + 1] = dym1 * gvi + dym2 * gvj;
        gw[q] = dxm1 * gwi + dxm2 * gwj;   gw[q + 1] = dym1 * gwi + dym2 * gwj;
        gmu[q] = dxm1 * gmui + dxm2 * gmuj; gmu[q + 1] = dym1 * gmui + dym2 * gmuj;
      }
  }
};

// coeffs_5p_dz (srcfv/dz/coeffs_5p_dz.F90:10-174): coefficients dz/coeffs_dz.F:1-97,
// functions matrix_dz/function_dz.F, sum dz/sum_coeffs_dz.F.  N directions; the
// interior of dz_out (N stacked padded arrays) is written, the ghosts are not.
template <int N>
void coeffs_5p_dz(double* dz_out, const double* w, const double* wd, const double* nx, const double* ny,
                  const double* vol, int gh, const Consts& k, int im, int jm) {
  const int ni = im + 2 * gh, nj = jm + 2 * gh;
  const size_t n = (size_t)ni * nj * 5;
  std::vector<Dual<N>> wdl(n);
  for (size_t q = 0; q < n; ++q) {
    wdl[q].v = w[q];
    for (int d = 0; d < N; ++d) wdl[q].d[d] = wd[(size_t)d * n + q];
  }
  const SpanFields<double> B(w, nx, ny, vol, gh, k, im, jm, true);
  const SpanFields<Dual<N>> D(wdl.data(), nx, ny, vol, gh, k, im, jm, true);
  FArr<const Dual<N>> W(wdl.data(), ni, nj, 1 - gh);
  const double ONE = 1.0, ZERO = 0.0, TWOTHIRD = 2.0 / 3.0;
  for (int j = 1; j <= jm; ++j)
    for (int i = 1; i <= im; ++i) {
      const size_t q = B.c(i, j), g = 2 * q;
      // base-flow coefficients, coeffs(e, kk) with kk = 1..16 (coeffs_dz.F)
      const double mu = B.mu[q], velx = B.velx[q], vely = B.vely[q], velz = B.velz[q];
      const double gu1 = B.gu[g], gv2 = B.gv[g + 1], gw1 = B.gw[g], gw2 = B.gw[g + 1];
      const double gmu1 = B.gmu[g], gmu2 = B.gmu[g + 1];
      double cf[5][16];
      for (int e = 0; e < 5; ++e)
        for (int kk = 0; kk < 16; ++kk) cf[e][kk] = (kk == 0) ? ONE : ZERO;
      cf[1][1] = TWOTHIRD * gmu1; cf[2][1] = TWOTHIRD * gmu2; cf[3][1] = -gmu1;
      cf[4][1] = TWOTHIRD * (gmu1 * velx + mu * gu1);
      cf[1][2] = TWOTHIRD * mu; cf[2][2] = TWOTHIRD * mu; cf[3][2] = -gmu2; cf[4][2] = TWOTHIRD * mu * velx;
      cf[3][3] = -mu; cf[4][3] = -(gmu1 * velz + mu * gw1);
      cf[4][4] = -(mu * velz);
      cf[4][5] = TWOTHIRD * (gmu2 * vely + mu * gv2);
      cf[4][6] = TWOTHIRD * mu * vely;
      cf[4][7] = -(gmu2 * velz + mu * gw2);
      cf[4][8] = -(mu * velz);
      cf[4][9] = -(mu * gw1);
      cf[4][10] = -velx;
      cf[4][11] = -(mu * gw2);
      cf[4][12] = -vely;
      cf[4][13] = TWOTHIRD * mu * (gu1 + gv2);
      cf[4][14] = TWOTHIRD * velz * (gu1 + gv2);
      cf[4][15] = TWOTHIRD * mu * velz;
      // auxiliary functions on duals (function_dz.F), fn[kk][e]
      const Dual<N> dmu = D.mu[q], dvx = D.velx[q], dvy = D.vely[q], dvz = D.velz[q], dp = D.p[q];
      const Dual<N> dgu1 = D.gu[g], dgv2 = D.gv[g + 1], dgw1 = D.gw[g], dgw2 = D.gw[g + 1];
      Dual<N> fn[16][5];
      fn[0][0] = W(i, j, 4);
      fn[0][1] = W(i, j, 2) * dvz - dmu * dgw1;
      fn[0][2] = W(i, j, 3) * dvz - dmu * dgw2;
      fn[0][3] = W(i, j, 4) * dvz + dp + TWOTHIRD * dmu * (dgu1 + dgv2);
      fn[0][4] = (W(i, j, 5) + dp) * dvz;
      fn[1][1] = dvz; fn[1][2] = dvz; fn[1][3] = dvx; fn[1][4] = dvz;
      fn[2][1] = dgw1; fn[2][2] = dgw2; fn[2][3] = dvy; fn[2][4] = dgw1;
      fn[3][3] = dgu1 + dgv2; fn[3][4] = dvx;
      fn[4][4] = dgu1;
      fn[5][4] = dvz;
      fn[6][4] = dgw2;
      fn[7][4] = dvy;
      fn[8][4] = dgv2;
      fn[9][4] = dvx;
      fn[10][4] = dmu * dgw1;
      fn[11][4] = dvy;
      fn[12][4] = dmu * dgw2;
      fn[13][4] = dvz;
      fn[14][4] = dmu;
      fn[15][4] = dgu1 + dgv2;
      // sum_coeffs_dz.F: left to right over kk
      for (int d = 0; d < N; ++d) {
        FArr<double> out(dz_out + (size_t)d * n, ni, nj, 1 - gh);
        for (int e = 0; e < 5; ++e) {
          double acc = cf[e][0] * fn[0][e].d[d];
          for (int kk = 1; kk < 16; ++kk) acc = acc + cf[e][kk] * fn[kk][e].d[d];
          out(i, j, e + 1) = acc;
        }
      }
    }
}

// coeffs_5p_dz2 (srcfv/dz/coeffs_5p_dz2.F90:10-147): coefficients dz/coeffs_dz2.F,
// functions matrix_dz2/function_dz2.F, sum dz/sum_coeffs_dz2.F.
template <int N>
void coeffs_5p_dz2(double* dz_out, const double* w, const double* wd, int gh, const Consts& k, int im, int jm) {
  const int ni = im + 2 * gh, nj = jm + 2 * gh;
  const size_t n = (size_t)ni * nj * 5;
  std::vector<Dual<N>> wdl(n);
  for (size_t q = 0; q < n; ++q) {
    wdl[q].v = w[q];
    for (int d = 0; d < N; ++d) wdl[q].d[d] = wd[(size_t)d * n + q];
  }
  const SpanFields<double> B(w, nullptr, nullptr, nullptr, gh, k, im, jm, false);
  const SpanFields<Dual<N>> D(wdl.data(), nullptr, nullptr, nullptr, gh, k, im, jm, false);
  const double TWO = 2.0, TWOTHIRD = 2.0 / 3.0, cpprandtl = k.cp / k.prandtl;
  for (int j = 1; j <= jm; ++j)
    for (int i = 1; i <= im; ++i) {
      const size_t q = B.c(i, j);
      const double mu = B.mu[q];
      double cf[5][4] = {};
      cf[1][0] = -mu; cf[2][0] = -mu; cf[3][0] = -(TWO * TWOTHIRD * mu); cf[4][0] = -(mu * cpprandtl);
      cf[4][1] = -(mu * B.velx[q]);
      cf[4][2] = -(mu * B.vely[q]);
      cf[4][3] = -(TWO * TWOTHIRD * mu * B.velz[q]);
      Dual<N> fn[4][5];
      fn[0][1] = D.velx[q]; fn[0][2] = D.vely[q]; fn[0][3] = D.velz[q]; fn[0][4] = D.tloc[q];
      fn[1][4] = D.velx[q]; fn[2][4] = D.vely[q]; fn[3][4] = D.velz[q];
      for (int d = 0; d < N; ++d) {
        FArr<double> out(dz_out + (size_t)d * n, ni, nj, 1 - gh);
        for (int e = 0; e < 5; ++e) {
          double acc = cf[e][0] * fn[0][e].d[d];
          for (int kk = 1; kk < 4; ++kk) acc = acc + cf[e][kk] * fn[kk][e].d[d];
          out(i, j, e + 1) = acc;
        }
      }
    }
}

// ===========================================================================
// Norms (srcfv/norm.F90)
// ===========================================================================
inline void compute_norml2(double* norm, double* nmoy, const double* rhs_, int im, int jm, int gh) {
  FArr<const double> rhs(rhs_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  double s[5] = {0, 0, 0, 0, 0};
  for (int j = 1; j <= jm; ++j)
    for (int i = 1; i <= im; ++i)
      for (int e = 1; e <= 5; ++e) s[e - 1] = s[e - 1] + rhs(i, j, e) * rhs(i, j, e);
  for (int e = 0; e < 5; ++e) { norm[e] = std::sqrt(s[e]); nmoy[e] = norm[e] / (double)(im * jm); }
}
inline void compute_norml2inf(double* norm, double* ninf, const double* rhs_, int im, int jm, int gh) {
  FArr<const double> rhs(rhs_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  double s[5] = {0, 0, 0, 0, 0}, t[5] = {0, 0, 0, 0, 0};
  for (int j = 1; j <= jm; ++j)
    for (int i = 1; i <= im; ++i)
      for (int e = 1; e <= 5; ++e) {
        s[e - 1] = s[e - 1] + rhs(i, j, e) * rhs(i, j, e);
        t[e - 1] = t[e - 1] + std::pow(rhs(i, j, e), 10.0);
      }
  for (int e = 0; e < 5; ++e) { norm[e] = std::sqrt(s[e]); ninf[e] = std::pow(t[e], 0.1); }
}
inline void compute_maxnorm(double* norm, int* imax, int* jmax, const double* rhs_, int im, int jm, int gh) {
  FArr<const double> rhs(rhs_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  for (int e = 0; e < 5; ++e) norm[e] = 0.0;
  for (int j = 1; j <= jm; ++j)
    for (int i = 1; i <= im; ++i)
      for (int e = 0; e < 5; ++e) {
        norm[e] = std::fabs(norm[e]);
        if (std::fabs(rhs(i, j, e + 1)) > norm[e]) { norm[e] = rhs(i, j, e + 1); imax[e] = i; jmax[e] = j; }
      }
}

// ===========================================================================
// Colored Jacobian assembly indexing (misc/ComputeJacobian.f90)
// ===========================================================================
// testvector (ComputeJacobian.f90:357-374)
inline void testvector(double* wd_, int m, int l, int k, int gh, int im, int jm) {
  FArr<double> wd(wd_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  const int step = 1 + 2 * gh;
  std::memset(wd_, 0, sizeof(double) * (size_t)(im + 2 * gh) * (jm + 2 * gh) * 5);
  for (int j = k + 1; j <= jm; j += step)
    for (int i = l + 1; i <= im; i += step) wd(i, j, m + 1) = 1.0;
}
// testvector_partial (ComputeJacobian.f90:1075-1092)
inline void testvector_partial(double* wd_, int m, int l, int k, int gh, int im, int jm, int istart, int iend,
                               int jstart, int jend) {
  FArr<double> wd(wd_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  const int step = 1 + 2 * gh;
  std::memset(wd_, 0, sizeof(double) * (size_t)(im + 2 * gh) * (jm + 2 * gh) * 5);
  for (int j = jstart + k + 1; j <= jend + 1; j += step)
    for (int i = istart + l + 1; i <= iend + 1; i += step) wd(i, j, m + 1) = 1.0;
}

// Variants of the COO fill.  mode selects the reference routine:
enum JacMode {
  JAC_PLAIN = 0,          // computejacobianfromjv            (:292-355)
  JAC_RELAXED = 1,        // computejacobianfromjv_relaxed    (:503-570)
  JAC_RELAXED_WITHJN = 2, // computejacobianfromjv_relaxed_withjn (:847-926)
  JAC_WITHJN = 3,         // computejacobianfromjv_withjn     (:929-999)
  JAC_DZ = 4,             // computejacobianfromdz            (:708-779)
};
// One COO slot of seed (m, l, k) for output (i, j, e): row, column and value,
// or the reference's invalid-slot marker (row 5*im*jm-1, or -2 for the _withjn
// variants; column 0, value 0).
inline void jacobian_slot(int mode, const FArr<const double>& resd, int i, int j, int e, int m, int l, int k, int gh,
                          int im, int jm, const double* coefdiag, int* ia_out, int* ja_out, double* val_out) {
  const int step = 1 + 2 * gh;
  const bool jn = (mode == JAC_RELAXED_WITHJN || mode == JAC_WITHJN);
  const bool relaxed = (mode == JAC_RELAXED || mode == JAC_RELAXED_WITHJN);
  const int bad = jn ? 5 * im * jm - 2 : 5 * im * jm - 1;
  const int ia = e - 1 + (j - 1) * 5 + (i - 1) * jm * 5;
  int valj, vali;
  if (mode == JAC_DZ) {
    if (k <= gh) valj = (j <= k + 1 + gh) ? k : (j - (k + 1) + gh) / step * step + k;
    else valj = (j <= k - gh) ? jm + 1 : (j - (k + 1) + gh) / step * step + k;
  } else {
    valj = (j <= k + 1 + gh) ? k : (j - gh - (k + 1) + 2 * gh) / step * step + k;
  }
  if (valj >= jm) { *ia_out = bad; *ja_out = 0; *val_out = 0.0; return; }
  if (l <= gh) vali = (i <= l + 1 + gh) ? l : (i - (l + 1) + gh) / step * step + l;
  else {
    if (i <= l - gh) vali = jn ? im - 1 - 2 * gh + l : im + 1;
    else vali = (i - (l + 1) + gh) / step * step + l;
  }
  if (vali >= im) {
    if (jn && vali - im <= gh - 1) vali = l;
    else { *ia_out = bad; *ja_out = 0; *val_out = 0.0; return; }
  }
  const int ja = m + valj * 5 + vali * jm * 5;
  const double r = resd(i, j, e);
  *ia_out = ia;
  *ja_out = ja;
  if (mode == JAC_DZ) *val_out = r;
  else if (relaxed && ia == ja) *val_out = coefdiag[(i - 1) + (size_t)(j - 1) * im] - r;
  else *val_out = -r;
}

inline void computejacobian(int mode, double* jac, int* ia, int* ja, const double* resd_, int m, int l, int k,
                            int gh, int im, int jm, const double* coefdiag) {
  FArr<const double> resd(resd_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  const int step = 1 + 2 * gh;
  for (int e = 1; e <= 5; ++e)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        const long long cur = (long long)(i - 1) + (long long)(j - 1) * im + (long long)(e - 1) * im * jm +
                              (long long)k * im * jm * 5 + (long long)l * im * jm * 5 * step +
                              (long long)m * im * jm * 5 * step * step;
        jacobian_slot(mode, resd, i, j, e, m, l, k, gh, im, jm, coefdiag, ia + cur, ja + cur, jac + cur);
      }
}

// The slots of one seed for the outputs of columns i0..i1 only, in a
// band-local layout: slot (i - i0) + (j - 1) nb + (e - 1) nb jm with
// nb = i1 - i0 + 1 (test infrastructure: the full COO of a large grid does not
// fit in memory, the slots of one seed and a band of rows do).
inline void computejacobian_band(int mode, double* jac, int* ia, int* ja, const double* resd_, int m, int l, int k,
                                 int gh, int im, int jm, const double* coefdiag, int i0, int i1) {
  FArr<const double> resd(resd_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  const long long nb = i1 - i0 + 1;
  for (int e = 1; e <= 5; ++e)
    for (int j = 1; j <= jm; ++j)
      for (int i = i0; i <= i1; ++i) {
        const long long cur = (long long)(i - i0) + (long long)(j - 1) * nb + (long long)(e - 1) * nb * jm;
        jacobian_slot(mode, resd, i, j, e, m, l, k, gh, im, jm, coefdiag, ia + cur, ja + cur, jac + cur);
      }
}

// computejacobianfromjv_relaxed_withjnandcheck (ComputeJacobian.f90:1095-1204)
inline void computejacobian_withjnandcheck(double* jac, int* ia, int* ja, const double* resd_, int m, int l, int k,
                                           int gh, int im, int jm, const double* coefdiag, double mini, int n) {
  FArr<const double> resd(resd_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  const int step = 1 + 2 * gh;
  const int bad = 5 * im * jm - 2;
  for (int e = 1; e <= 5; ++e)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        const long long cur = (long long)(i - 1) + (long long)(j - 1) * im + (long long)(e - 1) * im * jm +
                              (long long)k * im * jm * 5 + (long long)l * im * jm * 5 * step +
                              (long long)m * im * jm * 5 * step * step + (long long)n * im * jm * 5 * 5 * step * step;
        ia[cur] = e - 1 + (j - 1) * 5 + (i - 1) * jm * 5;
        const int valj = (j <= k + 1 + gh) ? k : (j - gh - (k + 1) + 2 * gh) / step * step + k;
        if (valj >= jm) { ia[cur] = bad; ja[cur] = 0; jac[cur] = 0.0; continue; }
        int vali;
        if (l <= gh) vali = (i <= l + 1 + gh) ? l : (i - (l + 1) + gh) / step * step + l;
        else vali = (i <= l - gh) ? l : (i - (l + 1) + gh) / step * step + l;
        const double cd = coefdiag[(i - 1) + (size_t)(j - 1) * im];
        const double r = resd(i, j, e);
        auto setv = [&](int vi) {
          ja[cur] = m + valj * 5 + vi * jm * 5;
          jac[cur] = (ia[cur] == ja[cur]) ? cd - r : -r;
        };
        if (n == 0) {
          if (vali >= im - 2 * gh) {
            vali = l;
            if (std::fabs(jac[cur]) < mini) setv(vali);
            else { ia[cur] = bad; ja[cur] = 0; jac[cur] = 0.0; }
          } else {
            if (std::fabs(jac[cur]) < mini) setv(vali);
          }
        } else {
          if (vali <= 2 * gh) {
            vali = im - (im % step) + l;
            if (vali > im - 1) vali = vali - step;
            if (std::fabs(jac[cur]) < mini) setv(vali);
          } else {
            if (std::fabs(jac[cur]) < mini) setv(vali);
            else { ia[cur] = bad; ja[cur] = 0; jac[cur] = 0.0; }
          }
        }
      }
}

// ===========================================================================
// Matrix-free implicit phase: srcfv/lhs/impli_matrix_free.F90:7-300
// (flattened srcfv/prepro/impli_matrix_free.f90).  lmax symmetric Gauss-Seidel
// sweeps (forward on odd l, backward on even l) of the scalar-diagonal
// implicit operator on the right-hand side dw; dwi returns the increment.
// ===========================================================================
inline void impli_matrix_free_2d(double* dwi_, const double* nx_, const double* ny_, const double* w_,
                                 const double* dw_, const double* vol_, const double* volf_, double dtcoef, double cfl,
                                 double gam, double rgaz, double prandtl, int lmax, int gh, double cv, double cs,
                                 double muref, double tref, double s_suth, int im, int jm) {
  const int ni = im + 2 * gh, nj = jm + 2 * gh, lo = 1 - gh;
  const size_t np = (size_t)ni * nj;
  FArr<double> dwi(dwi_, ni, nj, lo);
  FArr<const double> nx(nx_, ni + 1, nj + 1, lo), ny(ny_, ni + 1, nj + 1, lo), w(w_, ni, nj, lo),
      dw(dw_, ni, nj, lo), vol(vol_, ni, nj, lo), volf(volf_, ni, nj, lo);
  std::vector<double> tau0_(np), tloc_(np), mu_(np), d1w_(np * 5), f_(np * 5), g_(np * 5), ssor_(np * 5),
      coefdiag_(np), coef_(np * 2);
  FArr<double> tau0(tau0_.data(), ni, nj, lo), tloc(tloc_.data(), ni, nj, lo), mu(mu_.data(), ni, nj, lo),
      d1w(d1w_.data(), ni, nj, lo), f(f_.data(), ni, nj, lo), g(g_.data(), ni, nj, lo), ssor(ssor_.data(), ni, nj, lo),
      coefdiag(coefdiag_.data(), ni, nj, lo), coef(coef_.data(), ni, nj, lo);
  const double HALF = 0.5, ZERO = 0.0, TWO = 2.0, ONE = 1.0;
  for (size_t q = 0; q < np * 5; ++q) dwi_[q] = ZERO;
  const double gampr = 2.0 * gam / prandtl, gam1 = gam - ONE, cflm1 = ONE / cfl, cvm1 = ONE / cv;
  const double betas = muref * (tref + cs) / (std::sqrt(tref) * tref);
  (void)cflm1;
  // primitives, fluxes, viscosity and local time step on every padded cell
  // (lhs/PrimitivesLhs.F, phys/viscosity.F, lhs/time_step.F)
  for (int j = lo; j <= jm + gh; ++j)
    for (int i = lo; i <= im + gh; ++i) {
      const double ror = w(i, j, 1), rom1 = ONE / ror;
      const double velxi = w(i, j, 2) * rom1, velyi = w(i, j, 3) * rom1, velzi = w(i, j, 4) * rom1;
      const double ec = HALF * (velxi * velxi + velyi * velyi + velzi * velzi);
      const double eloc = (w(i, j, 5) - ec * ror) * rom1;
      tloc(i, j) = eloc * cvm1;
      const double pint = ror * rgaz * tloc(i, j);
      const double htot = (w(i, j, 5) + pint) * rom1;
      f(i, j, 1) = w(i, j, 2); f(i, j, 2) = w(i, j, 2) * velxi + pint; f(i, j, 3) = w(i, j, 2) * velyi;
      f(i, j, 4) = w(i, j, 2) * velzi; f(i, j, 5) = w(i, j, 2) * htot;
      g(i, j, 1) = w(i, j, 3); g(i, j, 2) = w(i, j, 3) * velxi; g(i, j, 3) = w(i, j, 3) * velyi + pint;
      g(i, j, 4) = w(i, j, 3) * velzi; g(i, j, 5) = w(i, j, 3) * htot;
      mu(i, j) = betas / (tloc(i, j) + s_suth) * std::sqrt(tloc(i, j)) * tloc(i, j);
      const double dist = vol(i, j) / (std::sqrt(nx(i, j, 1) * nx(i, j, 1) + ny(i, j, 1) * ny(i, j, 1)) +
                                       std::sqrt(nx(i, j, 2) * nx(i, j, 2) + ny(i, j, 2) * ny(i, j, 2)));
      const double cc = std::sqrt(gam * pint * rom1);
      const double vitc = std::sqrt(velxi * velxi + velyi * velyi) + cc;
      const double dt_euler = dist / vitc;
      const double dt_ns = 2.0 * dist * dist * ror / (gampr * mu(i, j));
      const double dt = std::max(std::min(dt_euler, dt_ns), 1e-15) * cfl;
      tau0(i, j) = dt / vol(i, j);
    }
  // face spectral radii, convective plus viscous (lhs/specrad_ns.F)
  for (int kdir = 1; kdir <= 2; ++kdir) {
    const int i0 = -kdir + 2, j0 = kdir - 1;
    for (int j = 1; j <= jm + j0; ++j)
      for (int i = 1; i <= im + i0; ++i) {
        const double rol = w(i - i0, j - j0, 1), ror = w(i, j, 1);
        const double rom1l = ONE / rol, rom1r = ONE / ror, iro = 2.0 / (rol + ror);
        const double uu = HALF * (w(i - i0, j - j0, 2) * rom1l + w(i, j, 2) * rom1r);
        const double vv = HALF * (w(i - i0, j - j0, 3) * rom1l + w(i, j, 3) * rom1r);
        const double cc = gam * rgaz * HALF * (tloc(i - i0, j - j0) + tloc(i, j));
        const double norm = nx(i, j, kdir) * nx(i, j, kdir) + ny(i, j, kdir) * ny(i, j, kdir);
        const double mutot = HALF * gampr * (mu(i - i0, j - j0) + mu(i, j));
        const double specdiff = mutot * norm * volf(i, j, kdir) * iro;
        coef(i, j, kdir) = ONE * (std::fabs(uu * nx(i, j, kdir) + vv * ny(i, j, kdir)) + std::sqrt(cc * norm) +
                                  TWO * specdiff);
      }
  }
  for (int j = 1; j <= jm; ++j)
    for (int i = 1; i <= im; ++i) {
      coefdiag(i, j) = tau0(i, j) * (coef(i, j, 1) + coef(i + 1, j, 1) + coef(i, j, 2) + coef(i, j + 1, 2)) + dtcoef;
      for (int e = 1; e <= 5; ++e) d1w(i, j, e) = dw(i, j, e) * tau0(i, j);
    }
  // lmax sweeps
  for (int l = 1; l <= lmax; ++l) {
    const double step = (l % 2 == 1) ? 1.0 : -1.0;  // (-1)**(l-1)
    const int ipas = (l % 2 == 1) ? 1 : -1;
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i)
        for (int e = 1; e <= 5; ++e) { dwi(i, j, e) = d1w(i, j, e) + ssor(i, j, e); ssor(i, j, e) = ZERO; }
    for (int jj = 0; jj < jm; ++jj)
      for (int ii = 0; ii < im; ++ii) {
        const int i = ipas > 0 ? 1 + ii : im - ii, j = ipas > 0 ? 1 + jj : jm - jj;
        double d2w[5] = {ZERO, ZERO, ZERO, ZERO, ZERO};
        for (int kdir = 1; kdir <= 2; ++kdir) {
          const int i0 = ipas * (-kdir + 2), j0 = ipas * (kdir - 1);
          const int ip = i - i0, jp = j - j0;
          const int irspec = i - i0 * (1 - ipas) / 2, jrspec = j - j0 * (1 - ipas) / 2;
          const double nxloc = nx(irspec, jrspec, kdir), nyloc = ny(irspec, jrspec, kdir);
          double wi[5], fi[5], gi[5];
          for (int e = 1; e <= 5; ++e) wi[e - 1] = w(ip, jp, e) + dwi(ip, jp, e);
          const double rhom1 = ONE / wi[0];
          const double velxi = wi[1] * rhom1, velyi = wi[2] * rhom1, velzi = wi[3] * rhom1;
          const double pint = gam1 * (wi[4] - HALF * wi[0] * (velxi * velxi + velyi * velyi + velzi * velzi));
          fi[0] = wi[1]; fi[1] = wi[1] * velxi + pint; fi[2] = wi[1] * velyi; fi[3] = wi[1] * velzi;
          fi[4] = velxi * (wi[4] + pint);
          gi[0] = wi[2]; gi[1] = wi[2] * velxi; gi[2] = wi[2] * velyi + pint; gi[3] = wi[2] * velzi;
          gi[4] = velyi * (wi[4] + pint);
          const double multi = HALF * step, multi2 = coef(irspec, jrspec, kdir);
          for (int e = 1; e <= 5; ++e) {
            const double dfi = fi[e - 1] - f(ip, jp, e), dgi = gi[e - 1] - g(ip, jp, e);
            d2w[e - 1] = d2w[e - 1] + multi * (dfi * nxloc + dgi * nyloc) + multi2 * dwi(ip, jp, e);
          }
        }
        const double cdiagm1 = ONE / coefdiag(i, j);
        for (int e = 1; e <= 5; ++e) {
          d2w[e - 1] = d2w[e - 1] * tau0(i, j);
          ssor(i, j, e) = d2w[e - 1] + ssor(i, j, e);
          dwi(i, j, e) = (d2w[e - 1] + dwi(i, j, e)) * cdiagm1;
        }
      }
    // ghost rows and columns of dwi: zero-gradient copies between sweeps, zero after the last
    const bool last = (l == lmax);
    for (int e = 1; e <= 5; ++e) {
      for (int i = 1; i <= im; ++i) dwi(i, jm + 1, e) = last ? ZERO : dwi(i, jm, e);
      for (int i = 1; i <= im; ++i) dwi(i, 0, e) = last ? ZERO : dwi(i, 1, e);
      for (int j = 1; j <= jm; ++j) dwi(im + 1, j, e) = last ? ZERO : dwi(im, j, e);
      for (int j = 1; j <= jm; ++j) dwi(0, j, e) = last ? ZERO : dwi(1, j, e);
    }
  }
}

// ===========================================================================
// Initial state helpers (initialisation.f90:2-58, set_bnd.f90:1-24)
// ===========================================================================
inline void initblfv(double muinf, const double* xc_, const double* yc_, double* w_, double* field_, int im, int gh,
                     int jm) {
  FArr<const double> xc(xc_, im + 2 * gh, jm + 2 * gh, 1 - gh), yc(yc_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  FArr<double> w(w_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  auto field = [&](int a, int b, int v) -> double& { return field_[(size_t)(a - 1) + (size_t)(b - 1) * jm + (size_t)(v - 1) * jm * gh]; };
  const double ro = w(3, 3, 1), rou = w(3, 3, 2), roE = w(3, 3, 5);
  const double ue = rou / ro, rou2 = 0.5 * rou * ue, xdeltam1 = std::sqrt(rou / muinf);
  for (int j = 1; j <= jm + gh; ++j)
    for (int i = 1 - gh; i <= im + gh; ++i) {
      const double eta = yc(i, j) * xdeltam1 / std::sqrt(xc(i, j));
      double ubl = (eta < 1.0) ? 2.0 * eta - 2.0 * eta * eta * eta + eta * eta * eta * eta : 1.0;
      ubl = ubl * ue;
      w(i, j, 2) = ro * ubl;
      w(i, j, 5) = roE - rou2 + 0.5 * ro * ubl * ubl;
    }
  for (int i = 1 - gh; i <= im + gh; ++i) w(i, 0, 2) = -w(i, 1, 2);
  for (int j = 1; j <= jm; ++j)
    for (int i = 1 - gh; i <= 0; ++i) {
      const double eta = yc(i, j) * xdeltam1 * std::sqrt(xc(i, j));
      double ubl = (eta < 1.0) ? 2.0 * eta - 2.0 * eta * eta * eta + eta * eta * eta * eta : 1.0;
      ubl = ubl * ue;
      field(j, 1 - i, 2) = ro * ubl;
      field(j, 1 - i, 5) = roE - rou2 + 0.5 * ro * ubl * ubl;
    }
}
inline void set_bndbl_2d(const double* w_, double* field_, double* wbd_, int im, int jm, int gh) {
  FArr<const double> w(w_, im + 2 * gh, jm + 2 * gh, 1 - gh);
  for (int j = 1; j <= jm; ++j)
    for (int d = 1; d <= gh; ++d)
      for (int v = 1; v <= 5; ++v) field_[(size_t)(j - 1) + (size_t)(d - 1) * jm + (size_t)(v - 1) * jm * gh] = w(1 - d, j, v);
  const int lm = im + gh;
  for (int i = 1; i <= im + gh; ++i)
    for (int v = 1; v <= 5; ++v) wbd_[(size_t)(i - 1) + (size_t)(v - 1) * lm] = w(i - gh, jm, v);
}

}  // namespace orc
