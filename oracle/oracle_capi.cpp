// Test infrastructure only: C entry points of the CPU oracle (liboracle.so).
// Loaded by tests/, __graft_entry__.smoke() and the cpu_baseline leg of
// bench.py through ctypes; never linked into the product library.
//
// Argument order follows the reference's f2py routines (see the citation on
// each function in broadcast_oracle.hpp); the unused x0,y0,xc,yc arguments of
// the residual are dropped here.
#include <algorithm>
#include <cstdlib>
#include <vector>
#include "broadcast_oracle.hpp"

using namespace orc;

namespace {
Consts mk(double cp, double cv, double prandtl, double gam, double rgaz, double cs, double muref, double tref,
          double s_suth, double k2, double k4) {
  Consts c;
  c.cp = cp; c.cv = cv; c.prandtl = prandtl; c.gam = gam; c.rgaz = rgaz; c.cs = cs; c.muref = muref;
  c.tref = tref; c.s_suth = s_suth; c.k2 = k2; c.k4 = k4;
  return c;
}
inline size_t np_(int im, int jm, int gh) { return (size_t)(im + 2 * gh) * (jm + 2 * gh); }

template <int K>
void jvp_k(double* res, double* resd, const double* w, const double* wd, int nd, const double* nx, const double* ny,
           const double* vol, const double* volf, int gh, const Consts& c, int im, int jm, bool wall = true,
           int order = 5) {
  const size_t n = np_(im, jm, gh) * 5;
  std::vector<Dual<K>> wdual(n), rdual(n);
  // wd holds nd <= K directions: the dual slots past nd stay zero (they are
  // never written back), so nothing past the caller's nd planes is read
  for (size_t q = 0; q < n; ++q) {
    wdual[q].v = w[q];
    for (int k = 0; k < K; ++k) wdual[q].d[k] = k < nd ? wd[(size_t)k * n + q] : 0.0;
  }
  flux_num_dnc5_2d<Dual<K>>(rdual.data(), wdual.data(), nx, ny, vol, volf, gh, c, im, jm, wall, order);
  FArr<Dual<K>> r(rdual.data(), im + 2 * gh, jm + 2 * gh, 1 - gh);
  FArr<double> rv(res, im + 2 * gh, jm + 2 * gh, 1 - gh);
  for (int e = 1; e <= 5; ++e)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) {
        if (res) rv(i, j, e) = r(i, j, e).v;
        for (int k = 0; k < nd; ++k) {
          FArr<double> rd(resd + (size_t)k * n, im + 2 * gh, jm + 2 * gh, 1 - gh);
          rd(i, j, e) = r(i, j, e).d[k];
        }
      }
}

template <class F>
void bc_dual(double* w, double* wd, size_t n, F&& body) {
  std::vector<Dual<1>> a(n);
  for (size_t q = 0; q < n; ++q) { a[q].v = w[q]; a[q].d[0] = wd[q]; }
  body(a.data());
  for (size_t q = 0; q < n; ++q) { w[q] = a[q].v; wd[q] = a[q].d[0]; }
}
}  // namespace

extern "C" {

// ---- residual ------------------------------------------------------------
int orc_flux_num_dnc5_2d(double* residu, const double* w, const double* nx, const double* ny, const double* vol,
                         const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz,
                         double cs, double muref, double tref, double s_suth, double k2, double k4, int im, int jm) {
  flux_num_dnc5_2d<double>(residu, w, nx, ny, vol, volf, gh, mk(cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4), im, jm);
  return 0;
}

// JVP for nd directions at once: wd and residud hold nd stacked padded arrays.
int orc_flux_num_dnc5_2d_d(double* residu, double* residud, const double* w, const double* wd, int nd,
                           const double* nx, const double* ny, const double* vol, const double* volf, int gh,
                           double cp, double cv, double prandtl, double gam, double rgaz, double cs, double muref,
                           double tref, double s_suth, double k2, double k4, int im, int jm) {
  const Consts c = mk(cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4);
  const size_t n = np_(im, jm, gh) * 5;
  for (int k0 = 0; k0 < nd; k0 += 8) {
    const int kk = std::min(8, nd - k0);
    double* r0 = (k0 == 0) ? residu : nullptr;
    if (kk == 1) jvp_k<1>(r0, residud + k0 * n, w, wd + k0 * n, 1, nx, ny, vol, volf, gh, c, im, jm);
    else if (kk <= 2) jvp_k<2>(r0, residud + k0 * n, w, wd + k0 * n, kk, nx, ny, vol, volf, gh, c, im, jm);
    else if (kk <= 4) jvp_k<4>(r0, residud + k0 * n, w, wd + k0 * n, kk, nx, ny, vol, volf, gh, c, im, jm);
    else jvp_k<8>(r0, residud + k0 * n, w, wd + k0 * n, kk, nx, ny, vol, volf, gh, c, im, jm);
  }
  return 0;
}

// ---- residual and JVP without the wall rows (flux_num_dnc5_nowall_2d) ----------
int orc_flux_num_dnc5_nowall_2d(double* residu, const double* w, const double* nx, const double* ny,
                                const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                                double gam, double rgaz, double cs, double muref, double tref, double s_suth,
                                double k2, double k4, int im, int jm) {
  flux_num_dnc5_2d<double>(residu, w, nx, ny, vol, volf, gh, mk(cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4),
                           im, jm, false);
  return 0;
}
int orc_flux_num_dnc5_nowall_2d_d(double* residu, double* residud, const double* w, const double* wd, int nd,
                                  const double* nx, const double* ny, const double* vol, const double* volf, int gh,
                                  double cp, double cv, double prandtl, double gam, double rgaz, double cs,
                                  double muref, double tref, double s_suth, double k2, double k4, int im, int jm) {
  const Consts c = mk(cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4);
  const size_t n = np_(im, jm, gh) * 5;
  for (int k0 = 0; k0 < nd; k0 += 4) {
    const int kk = std::min(4, nd - k0);
    jvp_k<4>(k0 == 0 ? residu : nullptr, residud + k0 * n, w, wd + k0 * n, kk, nx, ny, vol, volf, gh, c, im, jm,
             false);
  }
  return 0;
}

// ---- residual and JVP of the DNC schemes of order 3, 5, 7, 9, with or without
// the wall rows (flux_num_dnc{3,5,7,9}[_nowall]_2d[_d]) --------------------------
int orc_flux_num_dnc_2d(int order, int wall, double* residu, const double* w, const double* nx, const double* ny,
                        const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                        double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
                        double k4, int im, int jm) {
  if (dnc_coefs(order).order == 0 || gh < (order + 1) / 2) return -1;
  flux_num_dnc5_2d<double>(residu, w, nx, ny, vol, volf, gh, mk(cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4),
                           im, jm, wall != 0, order);
  return 0;
}
int orc_flux_num_dnc_2d_d(int order, int wall, double* residu, double* residud, const double* w, const double* wd,
                          int nd, const double* nx, const double* ny, const double* vol, const double* volf, int gh,
                          double cp, double cv, double prandtl, double gam, double rgaz, double cs, double muref,
                          double tref, double s_suth, double k2, double k4, int im, int jm) {
  if (dnc_coefs(order).order == 0 || gh < (order + 1) / 2) return -1;
  const Consts c = mk(cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4);
  const size_t n = np_(im, jm, gh) * 5;
  for (int k0 = 0; k0 < nd; k0 += 4) {
    const int kk = std::min(4, nd - k0);
    jvp_k<4>(k0 == 0 ? residu : nullptr, residud + k0 * n, w, wd + k0 * n, kk, nx, ny, vol, volf, gh, c, im, jm,
             wall != 0, order);
  }
  return 0;
}

// ---- matrix-free implicit phase (srcfv/lhs/impli_matrix_free.F90:7) ------------
int orc_impli_matrix_free_2d(double* dwi, const double* nx, const double* ny, const double* w, const double* dw,
                             const double* vol, const double* volf, double dtcoef, double cfl, double gam, double rgaz,
                             double prandtl, int lmax, int gh, double cv, double cs, double muref, double tref,
                             double s_suth, int im, int jm) {
  impli_matrix_free_2d(dwi, nx, ny, w, dw, vol, volf, dtcoef, cfl, gam, rgaz, prandtl, lmax, gh, cv, cs, muref, tref,
                       s_suth, im, jm);
  return 0;
}

// VJP: wb = (dR/dw)^T residub over every padded cell (the reference's
// adjoint/flux_num_dnc5_b.f90 overwrites wb and zeroes the interior of
// residub).  Computed exactly with Dual<5> sweeps over a period-9 colouring of
// the padded grid: a residual cell depends on cells at most 4 rows/columns
// away (3 in the interior; 4 through the near-wall j-fluxes of rows 2-3), so
// every residual cell sees at most one seeded cell per colour.
namespace {
int vjp_impl(double* residub, const double* w, double* wb, const double* nx, const double* ny, const double* vol,
             const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs,
             double muref, double tref, double s_suth, double k2, double k4, int im, int jm, bool wall);
}
int orc_flux_num_dnc5_2d_b(double* residub, const double* w, double* wb, const double* nx, const double* ny,
                           const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                           double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
                           double k4, int im, int jm) {
  return vjp_impl(residub, w, wb, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4,
                  im, jm, true);
}
// the same for the scheme without the wall rows (adjoint/flux_num_dnc5_nowall_b.f90)
int orc_flux_num_dnc5_nowall_2d_b(double* residub, const double* w, double* wb, const double* nx, const double* ny,
                                  const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                                  double gam, double rgaz, double cs, double muref, double tref, double s_suth,
                                  double k2, double k4, int im, int jm) {
  return vjp_impl(residub, w, wb, nx, ny, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4,
                  im, jm, false);
}
}  // extern "C"
namespace {
int vjp_impl(double* residub, const double* w, double* wb, const double* nx, const double* ny, const double* vol,
             const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs,
             double muref, double tref, double s_suth, double k2, double k4, int im, int jm, bool wall) {
  const Consts c = mk(cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4);
  const int ni = im + 2 * gh, nj = jm + 2 * gh, lo = 1 - gh;
  const size_t n = (size_t)ni * nj * 5;
  const int P = 9, R = 4;
  std::vector<Dual<5>> wdual(n), rdual(n);
  FArr<double> wbv(wb, ni, nj, lo);
  FArr<double> rb(residub, ni, nj, lo);
  for (size_t q = 0; q < n; ++q) wb[q] = 0.0;
  for (int a = 0; a < P; ++a)
    for (int b = 0; b < P; ++b) {
      for (size_t q = 0; q < n; ++q) { wdual[q] = Dual<5>(w[q]); }
      FArr<Dual<5>> wv(wdual.data(), ni, nj, lo);
      for (int j = lo; j <= jm + gh; ++j)
        for (int i = lo; i <= im + gh; ++i)
          if (((i - lo) % P) == a && ((j - lo) % P) == b)
            for (int v = 1; v <= 5; ++v) wv(i, j, v).d[v - 1] = 1.0;
      flux_num_dnc5_2d<Dual<5>>(rdual.data(), wdual.data(), nx, ny, vol, volf, gh, c, im, jm, wall);
      FArr<Dual<5>> rv(rdual.data(), ni, nj, lo);
      for (int j = lo; j <= jm + gh; ++j)
        for (int i = lo; i <= im + gh; ++i) {
          if (((i - lo) % P) != a || ((j - lo) % P) != b) continue;
          for (int jj = std::max(1, j - R); jj <= std::min(jm, j + R); ++jj)
            for (int ii = std::max(1, i - R); ii <= std::min(im, i + R); ++ii)
              for (int e = 1; e <= 5; ++e) {
                const double rbar = rb(ii, jj, e);
                if (rbar == 0.0) continue;
                for (int v = 1; v <= 5; ++v) wbv(i, j, v) += rbar * rv(ii, jj, e).d[v - 1];
              }
        }
    }
  for (int e = 1; e <= 5; ++e)
    for (int j = 1; j <= jm; ++j)
      for (int i = 1; i <= im; ++i) rb(i, j, e) = 0.0;
  return 0;
}
}  // namespace
extern "C" {

// Operation tallies of one residual evaluation by kind (OpKind in dual.hpp),
// written to counts[OP_NKIND]; returns the total.
long long orc_flux_num_dnc5_2d_opcount(long long* counts, const double* w, const double* nx, const double* ny,
                                       const double* vol, const double* volf, int gh, double cp, double cv,
                                       double prandtl, double gam, double rgaz, double cs, double muref, double tref,
                                       double s_suth, double k2, double k4, int im, int jm) {
  const Consts c = mk(cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4);
  const size_t n = np_(im, jm, gh) * 5;
  std::vector<OpCount> wo(n), ro(n);
  for (size_t q = 0; q < n; ++q) wo[q] = OpCount(w[q]);
  OpCount::reset();
  flux_num_dnc5_2d<OpCount>(ro.data(), wo.data(), nx, ny, vol, volf, gh, c, im, jm);
  long long tot = 0;
  for (int k = 0; k < OP_NKIND; ++k) { counts[k] = (long long)OpCount::tally()[k]; tot += counts[k]; }
  return tot;
}

// ---- boundary conditions ---------------------------------------------------
int orc_bc_wall_viscous_adia_2d(double* w, const char* loc, double gam, const int* interf, int gh, int im, int jm) {
  bc_wall_viscous_adia_2d<double>(w, loc, gam, interf, gh, im, jm);
  return 0;
}
int orc_bc_wall_viscous_adia_2d_d(double* w, double* wd, const char* loc, double gam, const int* interf, int gh,
                                  int im, int jm) {
  bc_dual(w, wd, np_(im, jm, gh) * 5, [&](Dual<1>* a) { bc_wall_viscous_adia_2d<Dual<1>>(a, loc, gam, interf, gh, im, jm); });
  return 0;
}
int orc_bc_no_reflexion_2d(double* w, const double* wbd, int lm, const char* loc, const int* interf, const double* nx,
                           const double* ny, double gam, int gh, int im, int jm) {
  bc_no_reflexion_2d<double>(w, wbd, lm, loc, interf, nx, ny, gam, gh, im, jm);
  return 0;
}
int orc_bc_no_reflexion_2d_d(double* w, double* wd, const double* wbd, int lm, const char* loc, const int* interf,
                             const double* nx, const double* ny, double gam, int gh, int im, int jm) {
  bc_dual(w, wd, np_(im, jm, gh) * 5, [&](Dual<1>* a) { bc_no_reflexion_2d<Dual<1>>(a, wbd, lm, loc, interf, nx, ny, gam, gh, im, jm); });
  return 0;
}
int orc_bc_supandsubinlet_2d(double* w, const char* loc, const int* interf, const double* field, int lm,
                             const double* nx, const double* ny, double gam, int im, int jm, int gh) {
  bc_supandsubinlet_2d<double>(w, loc, interf, field, lm, nx, ny, gam, im, jm, gh);
  return 0;
}
int orc_bc_supandsubinlet_2d_d(double* w, double* wd, const char* loc, const int* interf, const double* field,
                               int lm, const double* nx, const double* ny, double gam, int im, int jm, int gh) {
  bc_dual(w, wd, np_(im, jm, gh) * 5, [&](Dual<1>* a) { bc_supandsubinlet_2d<Dual<1>>(a, loc, interf, field, lm, nx, ny, gam, im, jm, gh); });
  return 0;
}
int orc_bc_extrapolate_o2_2d(double* w, const char* loc, const int* interf, int im, int jm, int gh, int em) {
  bc_extrapolate_o2_2d<double>(w, loc, interf, im, jm, gh, em);
  return 0;
}
int orc_bc_extrapolate_o2_2d_d(double* w, double* wd, const char* loc, const int* interf, int im, int jm, int gh,
                               int em) {
  const size_t n = np_(im, jm, gh) * em;
  std::vector<Dual<1>> a(n);
  for (size_t q = 0; q < n; ++q) { a[q].v = w[q]; a[q].d[0] = wd[q]; }
  bc_extrapolate_o2_2d<Dual<1>>(a.data(), loc, interf, im, jm, gh, em);
  for (size_t q = 0; q < n; ++q) { w[q] = a[q].v; wd[q] = a[q].d[0]; }
  return 0;
}
// ---- adjoints of the ghost fills (the reference's adjoint/bc_*_b.f90) ----------
// A fill writes the gh ghost layers of each boundary line from the line's
// positions 0..gh only, and lines are disjoint, so the transpose is exact from
// gh+1 Dual<5> runs, each seeding the 5 variables at one inward position p of
// every line:  wb(p) += sum over ghosts of d ghost / d w(p) * wb(ghost), then
// wb(ghosts) = 0.  kind: 0 wall, 1 no-reflexion, 2 inlet, 3 extrapolation.
int orc_bc_b(int kind, const double* w, double* wb, const double* aux, int lm, const char* loc, const int* interf,
             const double* nx, const double* ny, double gam, int gh, int im, int jm, int em) {
  const Side s(loc, interf);
  if (!s.ok) return -1;
  const int ni = im + 2 * gh, nj = jm + 2 * gh, lo = 1 - gh;
  const size_t n = (size_t)ni * nj * em;
  FArr<double> WB(wb, ni, nj, lo);
  std::vector<double> add(n, 0.0);
  FArr<double> ADD(add.data(), ni, nj, lo);
  for (int p = 0; p <= gh; ++p) {
    std::vector<Dual<5>> a(n);
    for (size_t q = 0; q < n; ++q) a[q] = Dual<5>(w[q]);
    FArr<Dual<5>> A(a.data(), ni, nj, lo);
    for (int l = s.lmin; l <= s.lmax; ++l)
      for (int v = 1; v <= em; ++v) A(s.li(l) + p * s.i0, s.lj(l) + p * s.j0, v).d[v - 1] = 1.0;
    if (kind == 0) bc_wall_viscous_adia_2d<Dual<5>>(a.data(), loc, gam, interf, gh, im, jm);
    else if (kind == 1) bc_no_reflexion_2d<Dual<5>>(a.data(), aux, lm, loc, interf, nx, ny, gam, gh, im, jm);
    else if (kind == 2) bc_supandsubinlet_2d<Dual<5>>(a.data(), loc, interf, aux, lm, nx, ny, gam, im, jm, gh);
    else bc_extrapolate_o2_2d<Dual<5>>(a.data(), loc, interf, im, jm, gh, em);
    for (int l = s.lmin; l <= s.lmax; ++l)
      for (int k = 1; k <= em; ++k) {
        double acc = 0.0;
        for (int q = 1; q <= gh; ++q)
          for (int v = 1; v <= em; ++v)
            acc += A(s.li(l) - q * s.i0, s.lj(l) - q * s.j0, v).d[k - 1] * WB(s.li(l) - q * s.i0, s.lj(l) - q * s.j0, v);
        ADD(s.li(l) + p * s.i0, s.lj(l) + p * s.j0, k) += acc;
      }
  }
  for (int l = s.lmin; l <= s.lmax; ++l)
    for (int q = 1; q <= gh; ++q)
      for (int v = 1; v <= em; ++v) WB(s.li(l) - q * s.i0, s.lj(l) - q * s.j0, v) = 0.0;
  for (size_t q = 0; q < n; ++q) wb[q] += add[q];
  return 0;
}

int orc_jn_match_2d(double* wr, const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr, int jmr,
                    const double* wd, const int* prd, int gh1d, int gh2d, int gh3d, int gh4d, int imd, int jmd,
                    const int* tr, int em) {
  jn_match_2d<double>(wr, prr, gh1r, gh2r, gh3r, gh4r, imr, jmr, wd, prd, gh1d, gh2d, gh3d, gh4d, imd, jmd, tr, em);
  return 0;
}

// ---- geometry, norms, initial state ---------------------------------------
int orc_computegeom_2d(double* x0, double* y0, double* nx, double* ny, double* xc, double* yc, double* vol,
                       double* volf, int im, int jm, int gh) {
  computegeom_2d(x0, y0, nx, ny, xc, yc, vol, volf, im, jm, gh);
  return 0;
}
int orc_compute_norml2(double* norm, double* nmoy, const double* rhs, int im, int jm, int gh) {
  compute_norml2(norm, nmoy, rhs, im, jm, gh);
  return 0;
}
int orc_compute_norml2inf(double* norm, double* ninf, const double* rhs, int im, int jm, int gh) {
  compute_norml2inf(norm, ninf, rhs, im, jm, gh);
  return 0;
}
int orc_compute_maxnorm(double* norm, int* imax, int* jmax, const double* rhs, int im, int jm, int gh) {
  compute_maxnorm(norm, imax, jmax, rhs, im, jm, gh);
  return 0;
}
int orc_initblfv(double muinf, const double* xc, const double* yc, double* w, double* field, int im, int gh, int jm) {
  initblfv(muinf, xc, yc, w, field, im, gh, jm);
  return 0;
}
int orc_set_bndbl_2d(const double* w, double* field, double* wbd, int im, int jm, int gh) {
  set_bndbl_2d(w, field, wbd, im, jm, gh);
  return 0;
}

// ---- colored assembly indexing ---------------------------------------------
// ---- spanwise operators (coeffs_5p_dz, coeffs_5p_dz2), nd stacked directions
int orc_coeffs_5p_dz(double* dz_out, const double* w, const double* wd, int nd, const double* nx, const double* ny,
                     const double* vol, int gh, double cp, double cv, double prandtl, double gam, double rgaz,
                     double cs, double muref, double tref, double s_suth, int im, int jm, int which) {
  const Consts c = mk(cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, 0.0, 0.0);
  const size_t n = np_(im, jm, gh) * 5;
  for (int k0 = 0; k0 < nd; k0 += 4) {
    const int kk = std::min(4, nd - k0);
    std::vector<double> buf((size_t)4 * n, 0.0), out((size_t)4 * n, 0.0);
    std::copy(wd + (size_t)k0 * n, wd + (size_t)(k0 + kk) * n, buf.begin());
    std::copy(dz_out + (size_t)k0 * n, dz_out + (size_t)(k0 + kk) * n, out.begin());
    if (which == 1) coeffs_5p_dz<4>(out.data(), w, buf.data(), nx, ny, vol, gh, c, im, jm);
    else coeffs_5p_dz2<4>(out.data(), w, buf.data(), gh, c, im, jm);
    std::copy(out.begin(), out.begin() + (size_t)kk * n, dz_out + (size_t)k0 * n);
  }
  return 0;
}

int orc_testvector(double* wd, int m, int l, int k, int gh, int im, int jm) {
  testvector(wd, m, l, k, gh, im, jm);
  return 0;
}
int orc_testvector_partial(double* wd, int m, int l, int k, int gh, int im, int jm, int istart, int iend, int jstart,
                           int jend) {
  testvector_partial(wd, m, l, k, gh, im, jm, istart, iend, jstart, jend);
  return 0;
}
int orc_computejacobian(int mode, double* jac, int* ia, int* ja, const double* resd, int m, int l, int k, int gh,
                        int im, int jm, const double* coefdiag) {
  computejacobian(mode, jac, ia, ja, resd, m, l, k, gh, im, jm, coefdiag);
  return 0;
}
int orc_computejacobian_band(int mode, double* jac, int* ia, int* ja, const double* resd, int m, int l, int k,
                              int gh, int im, int jm, const double* coefdiag, int i0, int i1) {
  if (i0 < 1 || i1 > im || i1 < i0) return -1;
  computejacobian_band(mode, jac, ia, ja, resd, m, l, k, gh, im, jm, coefdiag, i0, i1);
  return 0;
}

int orc_computejacobian_withjnandcheck(double* jac, int* ia, int* ja, const double* resd, int m, int l, int k, int gh,
                                       int im, int jm, const double* coefdiag, double mini, int n) {
  computejacobian_withjnandcheck(jac, ia, ja, resd, m, l, k, gh, im, jm, coefdiag, mini, n);
  return 0;
}

}  // extern "C"
