// Ghost-cell boundary fills (primal and fused primal + K-direction tangent).
//
// Reference: srcfv/borders/bc_wall_viscous.F90, bc_no_reflexion.F90,
// bc_supandsubinlet.F90, bc_extrapolate.F90, jn_match.F90 with the index
// set-up of borders/init_2d.F; tangents srcfv/tangent/bc_*_d.f90.
// One thread per boundary line l; the gh ghost layers of a line depend on each
// other (extrapolation from the previous layer), so a line is sequential.
#include "bc.h"
#include "dual.cuh"

namespace bcg {

template <class S> struct MState;
template <> struct MState<double> {
  double* __restrict__ v;
  size_t dstride;
  BCG_HD double get(size_t q) const { return v[q]; }
  BCG_HD void set(size_t q, double x) const { v[q] = x; }
};
template <int K> struct MState<DK<K>> {
  double* __restrict__ v;
  double* __restrict__ d;
  size_t dstride;
  BCG_HD DK<K> get(size_t q) const {
    DK<K> r; r.v = v[q];
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = d[(size_t)k * dstride + q];
    return r;
  }
  BCG_HD void set(size_t q, const DK<K>& x) const {
    v[q] = x.v;
#pragma unroll
    for (int k = 0; k < K; ++k) d[(size_t)k * dstride + q] = x.d[k];
  }
};

struct Grid {
  int im, jm, gh, ni, nj;
  size_t np;
  BCG_HD size_t c(int i, int j, int v) const {
    return (size_t)(i + gh - 1) + (size_t)(j + gh - 1) * ni + (size_t)(v - 1) * np;
  }
  BCG_HD size_t n(int i, int j, int d) const {
    return (size_t)(i + gh - 1) + (size_t)(j + gh - 1) * (ni + 1) + (size_t)(d - 1) * (ni + 1) * (nj + 1);
  }
};
static Grid mkgrid(int im, int jm, int gh) {
  Grid g; g.im = im; g.jm = jm; g.gh = gh; g.ni = im + 2 * gh; g.nj = jm + 2 * gh; g.np = (size_t)g.ni * g.nj;
  return g;
}

// Accessors the line bodies below read and write through:
// GAcc : the global state (and tangents) in HBM;
// LAcc : one boundary line held by the thread, positions p = -3..3 along the
//        inward normal, cell (ib + p i0, jb + p j0); used by the adjoint.
template <class S>
struct GAcc {
  Grid g;
  MState<S> w;
  BCG_HD S get(int i, int j, int v) const { return w.get(g.c(i, j, v)); }
  BCG_HD void set(int i, int j, int v, const S& x) const { w.set(g.c(i, j, v), x); }
};
template <int K>
struct LAcc {
  int ib, jb, i0, j0;
  DK<K> x[7][5];
  BCG_HD int pos(int i, int j) const { return (i - ib) * i0 + (j - jb) * j0 + 3; }
  BCG_HD DK<K> get(int i, int j, int v) const { return x[pos(i, j)][v - 1]; }
  BCG_HD void set(int i, int j, int v, const DK<K>& a) { x[pos(i, j)][v - 1] = a; }
};

// borders/bc_wall_viscous.F90:2-99
template <class S, class A>
BCG_HD void wall_line(const Grid& g, const BcSide& s, int l, double gam, A& w) {
  const int i = s.imin + (l - s.lmin) * s.j0 * s.j0, j = s.jmin + (l - s.lmin) * s.i0 * s.i0;
  const int i0 = s.i0, j0 = s.j0;
  const double gam1 = gam - 1.0, gami = 1.0 / gam, THIRD = 1.0 / 3.0;
  auto W = [&](int ii, int jj, int v) { return w.get(ii, jj, v); };
  const S roe = W(i, j, 1);
  S roem1 = 1.0 / roe;
  const S ue = W(i, j, 2) * roem1, ve = W(i, j, 3) * roem1, we = W(i, j, 4) * roem1;
  const S pe = gam1 * (W(i, j, 5) - 0.5 * roe * (ue * ue + ve * ve));
  const S roe1 = W(i + i0, j + j0, 1);
  const S roe1m1 = 1.0 / roe1;
  const S ue1 = W(i + i0, j + j0, 2) * roe1m1, ve1 = W(i + i0, j + j0, 3) * roe1m1;
  const S pe1 = gam1 * (W(i + i0, j + j0, 5) - 0.5 * roe1 * (ue1 * ue1 + ve1 * ve1));
  const S pw = 1.125 * pe + (-0.125) * pe1;
  const S pi = THIRD * (4.0 * pw - pe);
  S roi = pow_t(pi / pe * pow_t(roe, gam), gami);
  S ui = -ue, vi = -ve, wi = -we;
  S roiei = pi / gam1 + 0.5 * roi * (ui * ui + vi * vi);
  for (int de = 1; de <= g.gh; ++de) {
    w.set(i - de * i0, j - de * j0, 1, roi);
    w.set(i - de * i0, j - de * j0, 2, roi * ui);
    w.set(i - de * i0, j - de * j0, 3, roi * vi);
    w.set(i - de * i0, j - de * j0, 4, roi * wi);
    w.set(i - de * i0, j - de * j0, 5, roiei);
    roi = W(i + de * i0, j + de * j0, 1);
    roem1 = 1.0 / roi;
    const S a = W(i + de * i0, j + de * j0, 2) * roem1;
    const S b = W(i + de * i0, j + de * j0, 3) * roem1;
    const S cc = W(i + de * i0, j + de * j0, 4) * roem1;
    roiei = W(i + de * i0, j + de * j0, 5);
    ui = -a; vi = -b; wi = -cc;
  }
}

// borders/bc_no_reflexion.F90:8-152
template <class S, class A>
BCG_HD void noref_line(const Grid& g, const BcSide& s, int l, double gam, A& w, const double* __restrict__ wbd, int lm,
                       const double* __restrict__ nx, const double* __restrict__ ny) {
  const int i1 = s.i0 * s.i0, j1 = s.j0 * s.j0, i0 = s.i0, j0 = s.j0;
  const int i = s.imin + (l - s.lmin) * j1, j = s.jmin + (l - s.lmin) * i1;
  const double gam1 = gam - 1.0, sens = (double)(s.i0 + s.j0);
  auto W = [&](int ii, int jj, int v) { return w.get(ii, jj, v); };
  auto WBD = [&](int v) { return wbd[(size_t)(l - 1) + (size_t)(v - 1) * lm]; };
  const double nxloc = nx[g.n(i + s.high * i1, j + s.high * j1, s.kdir)];
  const double nyloc = ny[g.n(i + s.high * i1, j + s.high * j1, s.kdir)];
  const double nsumi = 1.0 / sqrt(nxloc * nxloc + nyloc * nyloc);
  const double nxn = nxloc * nsumi * sens, nyn = nyloc * nsumi * sens;
  const S ro0 = W(i, j, 1);
  const S ro0m1 = 1.0 / ro0;
  const S uu = W(i, j, 2) * ro0m1, vv = W(i, j, 3) * ro0m1, ww = W(i, j, 4) * ro0m1;
  const S p0 = gam1 * (W(i, j, 5) - 0.5 * ro0 * (uu * uu + vv * vv + ww * ww));
  const S roc0 = ro0 * sqrt_t(gam * p0 * ro0m1);
  const S roc0m1 = 1.0 / roc0;
  const S rovn0 = (W(i, j, 2) * nxn + W(i, j, 3) * nyn);
  const double epsm = 0.5 + fsign(0.5, roc0 - rovn0);
  const double eps0 = 0.5 + fsign(0.5, -rovn0);
  const double epsp = 0.5 + fsign(0.5, -roc0 - rovn0);
  const double rod = WBD(1), rodm1 = 1.0 / rod;
  const double ud = WBD(2) * rodm1, vd = WBD(3) * rodm1, wdi = WBD(4) * rodm1;
  const double pd = gam1 * (WBD(5) - rod * 0.5 * (ud * ud + vd * vd + wdi * wdi));
  const double vnd = (ud * nxn + vd * nyn);
  const double utd = ud - vnd * nxn, vtd = vd - vnd * nyn;
  const S ros = ro0, rosm1 = 1.0 / ros;
  const S us = W(i, j, 2) * rosm1, vs = W(i, j, 3) * rosm1, ws = W(i, j, 4) * rosm1;
  const S ps = gam1 * (W(i, j, 5) - ros * 0.5 * (us * us + vs * vs + ws * ws));
  const S vns = (us * nxn + vs * nyn);
  const S uts = us - vns * nxn, vts = vs - vns * nyn;
  const S ut = eps0 * uts + (1.0 - eps0) * utd;
  const S vt = eps0 * vts + (1.0 - eps0) * vtd;
  const S wt = eps0 * ws + (1.0 - eps0) * wdi;
  const S am = epsm * (ps - roc0 * vns) + (1.0 - epsm) * (pd - roc0 * vnd);
  const S ap = epsp * (ps + roc0 * vns) + (1.0 - epsp) * (pd + roc0 * vnd);
  const S vn = (ap - am) * 0.5 * roc0m1;
  const S pp = (ap + am) * 0.5;
  const S bs = (pp - ps) * ro0 * ro0 * roc0m1 * roc0m1 + ros;
  const S b0 = (pp - pd) * ro0 * ro0 * roc0m1 * roc0m1 + rod;
  S ro = eps0 * bs + (1.0 - eps0) * b0;
  const S rom1 = 1.0 / ro;
  const S roe = pp / gam1;
  S rou = ro * (ut + vn * nxn);
  S rov = ro * (vt + vn * nyn);
  S row = ro * wt;
  S roe2 = roe + 0.5 * rom1 * (rou * rou + rov * rov + row * row);
  for (int de = 1; de <= g.gh; ++de) {
    const int da = de - 1;
    w.set(i - de * i0, j - de * j0, 1, ro);
    w.set(i - de * i0, j - de * j0, 2, rou);
    w.set(i - de * i0, j - de * j0, 3, rov);
    w.set(i - de * i0, j - de * j0, 4, row);
    w.set(i - de * i0, j - de * j0, 5, roe2);
    ro = 2.0 * ro - W(i - da * i0, j - da * j0, 1);
    rou = 2.0 * rou - W(i - da * i0, j - da * j0, 2);
    rov = 2.0 * rov - W(i - da * i0, j - da * j0, 3);
    row = 2.0 * row - W(i - da * i0, j - da * j0, 4);
    roe2 = 2.0 * roe2 - W(i - da * i0, j - da * j0, 5);
  }
}

// borders/bc_supandsubinlet.F90:2-171 (reproduces the reference's factor on
// the Roe-state pressure and its velo2 = uu^2 + vv^2 + ww)
template <class S, class A>
BCG_HD void inlet_line(const Grid& g, const BcSide& s, int l, double gam, A& w, const double* __restrict__ field,
                       int lm, const double* __restrict__ nx, const double* __restrict__ ny) {
  const int i = s.imin + (l - s.lmin) * s.j0 * s.j0, j = s.jmin + (l - s.lmin) * s.i0 * s.i0;
  const int i0 = s.i0, j0 = s.j0;
  const double gam1 = gam - 1.0;
  auto W = [&](int ii, int jj, int v) { return w.get(ii, jj, v); };
  auto FLD = [&](int a, int b, int v) { return field[(size_t)(a - 1) + (size_t)(b - 1) * lm + (size_t)(v - 1) * lm * g.gh]; };
  const S wr1 = W(i, j, 1);
  S rom1 = 1.0 / wr1;
  const S wr2 = W(i, j, 2) * rom1, wr3 = W(i, j, 3) * rom1, wr4 = W(i, j, 4) * rom1;
  const S pr = gam1 * (W(i, j, 5) - wr1 * (wr2 * wr2 + wr3 * wr3 + wr4 * wr4));
  S hr = (W(i, j, 5) + pr) * rom1;
  const double wl1 = FLD(j, i, 1), rsm = 1.0 / wl1;
  const double wl2 = FLD(j, i, 2) * rsm, wl3 = FLD(j, i, 3) * rsm, wl4 = FLD(j, i, 4) * rsm;
  const double pl = gam1 * (FLD(j, i, 5) - wl1 * (wl2 * wl2 + wl3 * wl3 + wl4 * wl4));
  S hl = Planes<S>::c((FLD(j, i, 5) + pl) * rsm);
  S r = sqrt_t(wr1 / wl1);
  S rr = sqrt_t(wr1 * wl1);
  S oo = 1.0 / (r + 1.0);
  S uu = (wr2 * r + wl2) * oo, vv = (wr3 * r + wl3) * oo, ww = (wr4 * r + wl4) * oo;
  S hh = (hr * r + hl) * oo;
  const S velo2 = uu * uu + vv * vv + ww;
  S ee = 0.5 * velo2;
  S sound2 = gam1 * (hh - ee);
  const S mach = sqrt_t(velo2 / sound2);
  const bool sub = (mach < 1.0);
  double nxn = 0.0, nyn = 0.0, epsm = 0.0, eps0 = 0.0, epsp = 0.0;
  if (sub) {
    const double nxloc = nx[g.n(i, j, s.kdir)], nyloc = ny[g.n(i, j, s.kdir)];
    const double nsum = 1.0 / sqrt(nxloc * nxloc + nyloc * nyloc);
    nxn = nxloc * nsum; nyn = nyloc * nsum;
    const S roc0 = rr * sqrt_t(sound2);
    const S rovn0 = rr * (uu * nxn + vv * nyn);
    epsm = 0.5 + fsign(0.5, roc0 - rovn0);
    eps0 = 0.5 + fsign(0.5, -rovn0);
    epsp = 0.5 + fsign(0.5, -roc0 - rovn0);
  }
  for (int de = 1; de <= g.gh; ++de) {
#pragma unroll
    for (int v = 1; v <= 5; ++v) w.set(i - de * i0, j - de * j0, v, Planes<S>::c(FLD(l, de, v)));
    if (!sub) continue;
    const int da = de - 1;
    const S rod = W(i - de * i0, j - de * j0, 1);
    rom1 = 1.0 / rod;
    const S ud = W(i - de * i0, j - de * j0, 2) * rom1, vd = W(i - de * i0, j - de * j0, 3) * rom1;
    const S wd = W(i - de * i0, j - de * j0, 4) * rom1;
    const S pd = gam1 * (W(i - de * i0, j - de * j0, 5) - rod * 0.5 * (ud * ud + vd * vd + wd * wd));
    const S vnd = (ud * nxn + vd * nyn);
    const S utd = ud - vnd * nxn, vtd = vd - vnd * nyn;
    hl = (W(i - de * i0, j - de * j0, 5) + pd) * rom1;
    const S ros = W(i - da * i0, j - da * j0, 1);
    const S rosm1 = 1.0 / ros;
    const S us = W(i - da * i0, j - da * j0, 2) * rosm1, vs = W(i - da * i0, j - da * j0, 3) * rosm1;
    const S ws = W(i - da * i0, j - da * j0, 4) * rosm1;
    const S ps = gam1 * (W(i - da * i0, j - da * j0, 5) - ros * 0.5 * (us * us + vs * vs + ws * ws));
    const S vns = (us * nxn + vs * nyn);
    const S uts = us - vns * nxn, vts = vs - vns * nyn;
    hr = (W(i - da * i0, j - da * j0, 5) + ps) * rosm1;
    r = sqrt_t(ros * rom1);
    rr = sqrt_t(ros * rod);
    oo = 1.0 / (r + 1.0);
    uu = (us * r + ud) * oo; vv = (vs * r + vd) * oo; ww = (ws * r + wd) * oo;
    ee = 0.5 * (uu * uu + vv * vv + ww * ww);
    hh = (hr * r + hl) * oo;
    sound2 = gam1 * (hh - ee);
    const S roc0 = rr * sqrt_t(sound2);
    const S roc0m1 = 1.0 / roc0;
    const S ut = eps0 * uts + (1.0 - eps0) * utd;
    const S vt = eps0 * vts + (1.0 - eps0) * vtd;
    const S am = epsm * (ps - roc0 * vns) + (1.0 - epsm) * (pd - roc0 * vnd);
    const S ap = epsp * (ps + roc0 * vns) + (1.0 - epsp) * (pd + roc0 * vnd);
    const S vn = (ap - am) * 0.5 * roc0m1;
    const S pp = (ap + am) * 0.5;
    const S bs = (pp - ps) * rr * rr * roc0m1 * roc0m1 + ros;
    const S b0 = (pp - pd) * rr * rr * roc0m1 * roc0m1 + rod;
    const S ro = eps0 * bs + (1.0 - eps0) * b0;
    const S roe = pp / gam1;
    const S rou = ro * (ut + vn * nxn);
    const S rov = ro * (vt + vn * nyn);
    const S row = Planes<S>::c(FLD(j, de, 4));
    w.set(i - de * i0, j - de * j0, 1, ro);
    w.set(i - de * i0, j - de * j0, 2, rou);
    w.set(i - de * i0, j - de * j0, 3, rov);
    w.set(i - de * i0, j - de * j0, 4, row);
    w.set(i - de * i0, j - de * j0, 5, roe + 0.5 * (rou * rou + rov * rov + row * row) / ro);
  }
}

// borders/bc_extrapolate.F90:39-71
template <class S, class A>
BCG_HD void extrap_line(const Grid& g, const BcSide& s, int l, A& w, int em) {
  const int i = s.imin + (l - s.lmin) * s.j0 * s.j0, j = s.jmin + (l - s.lmin) * s.i0 * s.i0;
  for (int de = 1; de <= g.gh; ++de)
    for (int v = 1; v <= em; ++v) {
      const S a = w.get(i - s.i0 * (de - 1), j - s.j0 * (de - 1), v);
      const S b = w.get(i - s.i0 * (de - 2), j - s.j0 * (de - 2), v);
      w.set(i - s.i0 * de, j - s.j0 * de, v, 2.0 * a - b);
    }
}

// primal / tangent kernels: one thread per line on the global arrays
template <class S>
__global__ void k_bc_wall(Grid g, BcSide s, double gam, MState<S> w) {
  const int l = s.lmin + blockIdx.x * blockDim.x + threadIdx.x;
  if (l > s.lmax) return;
  GAcc<S> a{g, w};
  wall_line<S>(g, s, l, gam, a);
}
template <class S>
__global__ void k_bc_noref(Grid g, BcSide s, double gam, MState<S> w, const double* __restrict__ wbd, int lm,
                           const double* __restrict__ nx, const double* __restrict__ ny) {
  const int l = s.lmin + blockIdx.x * blockDim.x + threadIdx.x;
  if (l > s.lmax) return;
  GAcc<S> a{g, w};
  noref_line<S>(g, s, l, gam, a, wbd, lm, nx, ny);
}
template <class S>
__global__ void k_bc_inlet(Grid g, BcSide s, double gam, MState<S> w, const double* __restrict__ field, int lm,
                           const double* __restrict__ nx, const double* __restrict__ ny) {
  const int l = s.lmin + blockIdx.x * blockDim.x + threadIdx.x;
  if (l > s.lmax) return;
  GAcc<S> a{g, w};
  inlet_line<S>(g, s, l, gam, a, field, lm, nx, ny);
}
template <class S>
__global__ void k_bc_extrap(Grid g, BcSide s, MState<S> w, int em) {
  const int l = s.lmin + blockIdx.x * blockDim.x + threadIdx.x;
  if (l > s.lmax) return;
  GAcc<S> a{g, w};
  extrap_line<S>(g, s, l, a, em);
}

// Adjoint (srcfv/adjoint/bc_*_b.f90): a line writes its gh ghost layers from
// the values of its positions 0..gh (never from the ghosts' own input
// values), so per line  wb(0..gh) += J^T wb(ghosts), then wb(ghosts) = 0 for
// the written entries; w is left unchanged.  J (15 x 20) is taken column
// block by column block by running the line body on DK<5> numbers seeded on
// the 5 variables of one source position.  Lines are disjoint.
template <int KIND>
__global__ void k_bc_adj(Grid g, BcSide s, double gam, const double* __restrict__ w, double* __restrict__ wb,
                         const double* __restrict__ aux, int lm, const double* __restrict__ nx,
                         const double* __restrict__ ny, int em) {
  const int l = s.lmin + blockIdx.x * blockDim.x + threadIdx.x;
  if (l > s.lmax) return;
  const int i = s.imin + (l - s.lmin) * s.j0 * s.j0, j = s.jmin + (l - s.lmin) * s.i0 * s.i0;
  const int nv = (KIND == BC_EXTRAP) ? em : 5;
  double yb[3][5], xb[4][5];
  for (int q = 1; q <= 3; ++q)
    for (int v = 1; v <= 5; ++v) yb[q - 1][v - 1] = (v <= nv) ? wb[g.c(i - q * s.i0, j - q * s.j0, v)] : 0.0;
  for (int p = 0; p <= 3; ++p) {
    LAcc<5> a;
    a.ib = i; a.jb = j; a.i0 = s.i0; a.j0 = s.j0;
    for (int q = -3; q <= 3; ++q)
      for (int v = 1; v <= 5; ++v) {
        DK<5>& x = a.x[q + 3][v - 1];
        x.v = (v <= nv) ? w[g.c(i + q * s.i0, j + q * s.j0, v)] : 0.0;
#pragma unroll
        for (int k = 0; k < 5; ++k) x.d[k] = (q == p && k == v - 1) ? 1.0 : 0.0;
      }
    if (KIND == BC_WALL) wall_line<DK<5>>(g, s, l, gam, a);
    else if (KIND == BC_NOREF) noref_line<DK<5>>(g, s, l, gam, a, aux, lm, nx, ny);
    else if (KIND == BC_INLET) inlet_line<DK<5>>(g, s, l, gam, a, aux, lm, nx, ny);
    else extrap_line<DK<5>>(g, s, l, a, em);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      double acc = 0.0;
      for (int q = 1; q <= 3; ++q)
        for (int v = 1; v <= nv; ++v) acc += a.x[3 - q][v - 1].d[k] * yb[q - 1][v - 1];
      xb[p][k] = acc;
    }
  }
  for (int q = 1; q <= 3; ++q)
    for (int v = 1; v <= nv; ++v) wb[g.c(i - q * s.i0, j - q * s.j0, v)] = 0.0;
  for (int p = 0; p <= 3; ++p)
    for (int v = 1; v <= nv; ++v) wb[g.c(i + p * s.i0, j + p * s.j0, v)] += xb[p][v - 1];
}

// borders/jn_match.F90:3-66: block copy wr(ir,jr,:) = wd(id,jd,:).  One
// thread per copied cell.
__global__ void k_jn_match(JnArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.ncopy) return;
  const int ii = t % a.icount, jj = t / a.icount;   // 0-based offsets in loop order
  const int i = a.i1 + ii * a.istep, j = a.j1 + jj * a.jstep;
  const int ir = a.prr11 + ii, jr = a.prr12 + jj;
  const int id = a.prd1i + i - 1, jd = a.prd1j + j - 1;
  for (int v = 0; v < a.em; ++v)
    a.wr[(size_t)(ir - a.lor_i) + (size_t)(jr - a.lor_j) * a.nir + (size_t)v * a.nir * a.njr] =
        a.wd[(size_t)(id - a.lod_i) + (size_t)(jd - a.lod_j) * a.nid + (size_t)v * a.nid * a.njd];
}

// ---------------------------------------------------------------------------
template <class S>
static cudaError_t launch_bc_t(const BcArgs& a, cudaStream_t st) {
  const Grid g = mkgrid(a.im, a.jm, a.gh);
  const int n = a.side.lmax - a.side.lmin + 1;
  if (n <= 0) return cudaSuccess;
  const int B = 64;
  const unsigned nb = (unsigned)((n + B - 1) / B);
  MState<S> w;
  if constexpr (NDir<S>::value == 0) w = MState<S>{a.w, a.dstride};
  else w = MState<S>{a.w, a.wd, a.dstride};
  switch (a.kind) {
    case BC_WALL: k_bc_wall<S><<<nb, B, 0, st>>>(g, a.side, a.gam, w); break;
    case BC_NOREF: k_bc_noref<S><<<nb, B, 0, st>>>(g, a.side, a.gam, w, a.aux, a.lm, a.nx, a.ny); break;
    case BC_INLET: k_bc_inlet<S><<<nb, B, 0, st>>>(g, a.side, a.gam, w, a.aux, a.lm, a.nx, a.ny); break;
    case BC_EXTRAP: k_bc_extrap<S><<<nb, B, 0, st>>>(g, a.side, w, a.em); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_bc(const BcArgs& a, cudaStream_t st) {
  switch (a.ndir) {
    case 0: return launch_bc_t<double>(a, st);
    case 1: return launch_bc_t<DK<1>>(a, st);
    case 2: return launch_bc_t<DK<2>>(a, st);
    case 4: return launch_bc_t<DK<4>>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_bc_adjoint(const BcArgs& a, double* wb, cudaStream_t st) {
  if (a.gh != 3) return cudaErrorInvalidValue;  // LAcc holds positions -3..3
  const Grid g = mkgrid(a.im, a.jm, a.gh);
  const int n = a.side.lmax - a.side.lmin + 1;
  if (n <= 0) return cudaSuccess;
  const int B = 32;
  const unsigned nb = (unsigned)((n + B - 1) / B);
  switch (a.kind) {
    case BC_WALL: k_bc_adj<BC_WALL><<<nb, B, 0, st>>>(g, a.side, a.gam, a.w, wb, nullptr, 0, a.nx, a.ny, 5); break;
    case BC_NOREF: k_bc_adj<BC_NOREF><<<nb, B, 0, st>>>(g, a.side, a.gam, a.w, wb, a.aux, a.lm, a.nx, a.ny, 5); break;
    case BC_INLET: k_bc_adj<BC_INLET><<<nb, B, 0, st>>>(g, a.side, a.gam, a.w, wb, a.aux, a.lm, a.nx, a.ny, 5); break;
    case BC_EXTRAP: k_bc_adj<BC_EXTRAP><<<nb, B, 0, st>>>(g, a.side, a.gam, a.w, wb, nullptr, 0, a.nx, a.ny, a.em); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// adjoint of the block copy (adjoint/jn_match_2d_b.f90): wdb(donor) += wrb(receiver),
// wrb(receiver) = 0; the caller zeroes wdb first, as the reference does
__global__ void k_jn_match_b(JnArgs a, double* __restrict__ wrb, double* __restrict__ wdb) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.ncopy) return;
  const int ii = t % a.icount, jj = t / a.icount;
  const int i = a.i1 + ii * a.istep, j = a.j1 + jj * a.jstep;
  const int ir = a.prr11 + ii, jr = a.prr12 + jj;
  const int id = a.prd1i + i - 1, jd = a.prd1j + j - 1;
  for (int v = 0; v < a.em; ++v) {
    const size_t qr = (size_t)(ir - a.lor_i) + (size_t)(jr - a.lor_j) * a.nir + (size_t)v * a.nir * a.njr;
    const size_t qd = (size_t)(id - a.lod_i) + (size_t)(jd - a.lod_j) * a.nid + (size_t)v * a.nid * a.njd;
    const double x = wrb[qr];
    wrb[qr] = 0.0;
    wdb[qd] += x;
  }
}

cudaError_t launch_jn_match_adjoint(const JnArgs& a, double* wrb, double* wdb, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(wdb, 0, (size_t)a.nid * a.njd * a.em * sizeof(double), st);
  if (e != cudaSuccess || a.ncopy <= 0) return e;
  const int B = 128;
  k_jn_match_b<<<(a.ncopy + B - 1) / B, B, 0, st>>>(a, wrb, wdb);
  return cudaGetLastError();
}

cudaError_t launch_jn_match(const JnArgs& a, cudaStream_t st) {
  if (a.ncopy <= 0) return cudaSuccess;
  const int B = 128;
  k_jn_match<<<(a.ncopy + B - 1) / B, B, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace bcg
