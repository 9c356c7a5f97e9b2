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

}  // namespace bcg
