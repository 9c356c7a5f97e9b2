// Launch interface of the ghost-cell boundary kernels.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstring>

namespace bcg {

// Boundary side from the reference's loc string and interf(2,2) array
// (borders/init_2d.F).  interf in Fortran column-major order {imin, imax, jmin, jmax}.
struct BcSide {
  int kdir, i0, j0, high, lmin, lmax, imin, jmin, imax, jmax;
};
inline bool make_side(const char* loc, const int* interf, BcSide* s) {
  BcSide r{};
  r.imin = interf[0]; r.imax = interf[1]; r.jmin = interf[2]; r.jmax = interf[3];
  r.lmin = 1;
  if (!std::strncmp(loc, "Ilo", 3)) { r.kdir = 1; r.i0 = 1; r.lmax = r.jmax - r.jmin + 1; }
  else if (!std::strncmp(loc, "Ihi", 3)) { r.kdir = 1; r.i0 = -1; r.lmax = r.jmax - r.jmin + 1; r.high = 1; }
  else if (!std::strncmp(loc, "Jlo", 3)) { r.kdir = 2; r.j0 = 1; r.lmax = r.imax - r.imin + 1; }
  else if (!std::strncmp(loc, "Jhi", 3)) { r.kdir = 2; r.j0 = -1; r.lmax = r.imax - r.imin + 1; r.high = 1; }
  else return false;
  *s = r;
  return true;
}

// Every cell a line touches, base +- gh along the inward normal for l in
// [lmin, lmax], lies inside the padded (1-gh:im+gh, 1-gh:jm+gh) array.
inline bool side_in_bounds(const BcSide& s, int im, int jm, int gh) {
  if (s.lmax < s.lmin) return true;
  const int l1 = s.lmin, l2 = s.lmax;
  const int ia = s.imin + (l1 - s.lmin) * s.j0 * s.j0, ib = s.imin + (l2 - s.lmin) * s.j0 * s.j0;
  const int ja = s.jmin + (l1 - s.lmin) * s.i0 * s.i0, jb = s.jmin + (l2 - s.lmin) * s.i0 * s.i0;
  const int ilo = (ia < ib ? ia : ib) - gh * (s.i0 != 0), ihi = (ia > ib ? ia : ib) + gh * (s.i0 != 0);
  const int jlo = (ja < jb ? ja : jb) - gh * (s.j0 != 0), jhi = (ja > jb ? ja : jb) + gh * (s.j0 != 0);
  return ilo >= 1 - gh && ihi <= im + gh && jlo >= 1 - gh && jhi <= jm + gh;
}

enum BcKind { BC_WALL = 0, BC_NOREF = 1, BC_INLET = 2, BC_EXTRAP = 3 };

struct BcArgs {
  int kind, ndir, im, jm, gh, em, lm;
  BcSide side;
  double gam;
  double* w;            // (ni, nj, em) state, ghosts written
  double* wd;           // ndir stacked tangent states
  size_t dstride;
  const double* aux;    // wbd (lm,5) for BC_NOREF, field (lm,gh,5) for BC_INLET
  const double* nx;
  const double* ny;
};
cudaError_t launch_bc(const BcArgs& a, cudaStream_t st);
// adjoint of the fill: wb(positions 0..gh of each line) += J^T wb(ghosts),
// wb(written ghosts) = 0; a.w is read only (the primal state before the fill)
cudaError_t launch_bc_adjoint(const BcArgs& a, double* wb, cudaStream_t st);

struct JnArgs {
  double* wr;
  const double* wd;
  int em, ncopy, icount;
  int i1, istep, j1, jstep;
  int prr11, prr12, prd1i, prd1j;
  int lor_i, lor_j, nir, njr;   // receiver lower bounds and extents
  int lod_i, lod_j, nid, njd;   // donor lower bounds and extents
};
cudaError_t launch_jn_match(const JnArgs& a, cudaStream_t st);
// wdb = 0 over its whole extent, then wdb(donor) += wrb(receiver), wrb(receiver) = 0
cudaError_t launch_jn_match_adjoint(const JnArgs& a, double* wrb, double* wdb, cudaStream_t st);

}  // namespace bcg
