// Matrix-free implicit phase of the 'impli' time marching
// (srcfv/lhs/impli_matrix_free.F90:7-300, impli_matrix_free_2d): lmax
// symmetric Gauss-Seidel sweeps of the scalar-diagonal implicit operator
//   D dwi = tau0 dw - L/U(dwi),  forward on odd sweeps, backward on even ones,
// where each cell uses the fluxes of its already-updated upwind neighbours.
//
// GB300 layout of the work:
//   k_impli_cells / k_impli_faces / k_impli_diag  the sweep-invariant terms
//       (fluxes, local time step, face spectral radii, diagonal), one thread
//       per cell or face, in parallel, packed per cell into a 16-byte-aligned
//       record (CellRec) so that a sweep fetches a cell with a few 16-byte
//       copies;
//   k_impli_sweeps  all sweeps in ONE launch of one thread-block cluster.  A
//       Gauss-Seidel sweep is a wavefront: cell (i,j) needs (i-1,j) and
//       (i,j-1) of the same sweep (forward; (i+1,j), (i,j+1) backward), so the
//       cells of one anti-diagonal i + j = s are independent.  One thread owns
//       one grid row j and takes its cell (s-j, j) at step s; the rows are
//       split evenly over the cluster's CTAs (as many SMs' FP64 pipes), with
//       the hardware cluster barrier between steps instead of one launch per
//       diagonal.  Each updated cell forms its two flux terms for the
//       downstream faces once (the reference recomputes the upwind flux in
//       each consumer): the term along i stays in the thread's registers for
//       its next cell, the term along j goes to a shared-memory slot that the
//       neighbouring row reads at the next step (through distributed shared
//       memory across a CTA boundary).  A thread streams its next cells'
//       records into its own shared-memory ring with cp.async two steps
//       ahead, and the barrier is split (arrive after the slot write, wait at
//       the next step), so no global load sits on the critical path.  The
//       ghost neighbours of the first row and column are the reference's
//       zero-gradient copies, i.e. the previous sweep's values of the adjacent
//       interior cells; a row's first cell of a sweep is its last of the
//       previous one, whose values the thread still holds in registers.
//       Every cell combines the same terms in the reference's order, so the
//       result is the reference's Gauss-Seidel iterate, not a reordering.
//   k_impli_out  the increments into dwi (ghosts stay zero).
#include <mutex>
#include <cooperative_groups.h>
#include <cstdint>
#include "dnc5.cuh"
#include "impli.h"

namespace bcg {
namespace {

// per-cell record of the sweep-invariant terms (doubles); every padded cell
// has w, f, g, interior cells the rest.  Faces: "fwd" (i+1,j) along i and
// (i,j+1) along j, "bwd" (i,j) along i and (i,j) along j, each nx, ny, coef.
enum CellRec { C_W = 0, C_F = 5, C_G = 10, C_TAU0 = 15, C_CDM1 = 16, C_D1W = 17, C_FWD = 22, C_BWD = 28,
               C_NREC = 34 };
// per-cell carry (doubles): dwi, then the sweep carry-over (ssor)
enum CarryRec { K_DWI = 0, K_SSOR = 5, K_NREC = 10 };
// SoA planes used while building the records
enum ImpliPlane { I_TLOC = 0, I_MU = 1, I_COEF = 2, I_NPLANE = 4 };

struct ImpliK {
  Ext e;
  int lmax;
  double dtcoef, cfl, gam, rgaz, gampr, gam1, cvm1, betas, s_suth;
  const double* __restrict__ nx;
  const double* __restrict__ ny;
  const double* __restrict__ w;
  const double* __restrict__ dw;
  const double* __restrict__ vol;
  const double* __restrict__ volf;
  double* dwi;
  double* rec;    // np * C_NREC
  double* carry;  // np * K_NREC
  double* gterm;  // ghost-face terms of the current sweep: 6 per row, then 10 per column
  double* sc;     // I_NPLANE planes of np
  BCG_HD double* P(int plane) const { return sc + (size_t)plane * e.np; }
  BCG_HD size_t NI(int i, int j, int d) const { return (size_t)(d - 1) * e.nn() + e.nidx(i, j); }
};

// primitives, fluxes, viscosity and local time step of every padded cell
// (lhs/PrimitivesLhs.F, phys/viscosity.F, lhs/time_step.F); dwi and the carry
// start at zero
__global__ void __launch_bounds__(256) k_impli_cells(ImpliK k) {
  const Ext& e = k.e;
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= e.np) return;
  const int i = (int)(q % e.ni) + 1 - e.gh, j = (int)(q / e.ni) + 1 - e.gh;
  const size_t n = e.np;
  const double* w = k.w;
  const double ror = w[q], rom1 = 1.0 / ror;
  const double w2 = w[q + n], w3 = w[q + 2 * n], w4 = w[q + 3 * n], w5 = w[q + 4 * n];
  const double velxi = w2 * rom1, velyi = w3 * rom1, velzi = w4 * rom1;
  const double ec = 0.5 * (velxi * velxi + velyi * velyi + velzi * velzi);
  const double eloc = (w5 - ec * ror) * rom1;
  const double tloc = eloc * k.cvm1;
  const double pint = ror * k.rgaz * tloc;
  const double htot = (w5 + pint) * rom1;
  double* r = k.rec + q * C_NREC;
  r[C_W] = ror; r[C_W + 1] = w2; r[C_W + 2] = w3; r[C_W + 3] = w4; r[C_W + 4] = w5;
  r[C_F] = w2; r[C_F + 1] = w2 * velxi + pint; r[C_F + 2] = w2 * velyi; r[C_F + 3] = w2 * velzi; r[C_F + 4] = w2 * htot;
  r[C_G] = w3; r[C_G + 1] = w3 * velxi; r[C_G + 2] = w3 * velyi + pint; r[C_G + 3] = w3 * velzi; r[C_G + 4] = w3 * htot;
  const double mu = k.betas / (tloc + k.s_suth) * sqrt(tloc) * tloc;
  k.P(I_TLOC)[q] = tloc;
  k.P(I_MU)[q] = mu;
  const double n1x = k.nx[k.NI(i, j, 1)], n1y = k.ny[k.NI(i, j, 1)];
  const double n2x = k.nx[k.NI(i, j, 2)], n2y = k.ny[k.NI(i, j, 2)];
  const double volq = k.vol[q];
  const double dist = volq / (sqrt(n1x * n1x + n1y * n1y) + sqrt(n2x * n2x + n2y * n2y));
  const double cc = sqrt(k.gam * pint * rom1);
  const double vitc = sqrt(velxi * velxi + velyi * velyi) + cc;
  const double dt_euler = dist / vitc;
  const double dt_ns = 2.0 * dist * dist * ror / (k.gampr * mu);
  const double dt = fmax(fmin(dt_euler, dt_ns), 1e-15) * k.cfl;
  r[C_TAU0] = dt / volq;
  double* c = k.carry + q * K_NREC;
#pragma unroll
  for (int v = 0; v < K_NREC; ++v) c[v] = 0.0;
#pragma unroll
  for (int v = 0; v < 5; ++v) k.dwi[q + v * n] = 0.0;
}

// face spectral radii, convective plus viscous (lhs/specrad_ns.F): i-face
// (i,j) for i in [1, im+1], j in [1, jm]; j-face for i in [1, im], j in [1, jm+1]
__global__ void __launch_bounds__(256) k_impli_faces(ImpliK k) {
  const Ext& e = k.e;
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= e.np) return;
  const int i = (int)(q % e.ni) + 1 - e.gh, j = (int)(q / e.ni) + 1 - e.gh;
  const double* w = k.w;
  const size_t n = e.np;
  const double* tl = k.P(I_TLOC);
  const double* mu = k.P(I_MU);
#pragma unroll
  for (int kdir = 1; kdir <= 2; ++kdir) {
    const int i0 = 2 - kdir, j0 = kdir - 1;
    if (i < 1 || i > e.im + i0 || j < 1 || j > e.jm + j0) continue;
    const size_t ql = e.cidx(i - i0, j - j0);
    const double rol = w[ql], ror = w[q];
    const double rom1l = 1.0 / rol, rom1r = 1.0 / ror, iro = 2.0 / (rol + ror);
    const double uu = 0.5 * (w[ql + n] * rom1l + w[q + n] * rom1r);
    const double vv = 0.5 * (w[ql + 2 * n] * rom1l + w[q + 2 * n] * rom1r);
    const double cc = k.gam * k.rgaz * 0.5 * (tl[ql] + tl[q]);
    const double fnx = k.nx[k.NI(i, j, kdir)], fny = k.ny[k.NI(i, j, kdir)];
    const double norm = fnx * fnx + fny * fny;
    const double mutot = 0.5 * k.gampr * (mu[ql] + mu[q]);
    const double specdiff = mutot * norm * k.volf[q + (size_t)(kdir - 1) * n] * iro;
    k.P(I_COEF + kdir - 1)[q] = fabs(uu * fnx + vv * fny) + sqrt(cc * norm) + 2.0 * specdiff;
  }
}

// the diagonal (its reciprocal), the scaled right-hand side and the four
// faces of interior cell t
__global__ void __launch_bounds__(256) k_impli_diag(ImpliK k) {
  const Ext& e = k.e;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.im * e.jm) return;
  const int i = 1 + t % e.im, j = 1 + t / e.im;
  const size_t q = e.cidx(i, j), n = e.np;
  const double* c1 = k.P(I_COEF);
  const double* c2 = k.P(I_COEF + 1);
  double* r = k.rec + q * C_NREC;
  const double tau0 = r[C_TAU0];
  const double coefdiag = tau0 * (c1[q] + c1[q + 1] + c2[q] + c2[q + e.ni]) + k.dtcoef;
  r[C_CDM1] = 1.0 / coefdiag;
#pragma unroll
  for (int v = 0; v < 5; ++v) r[C_D1W + v] = k.dw[q + v * n] * tau0;
  auto face = [&](double* dst, int fi, int fj, int kdir) {
    dst[0] = k.nx[k.NI(fi, fj, kdir)];
    dst[1] = k.ny[k.NI(fi, fj, kdir)];
    dst[2] = k.P(I_COEF + kdir - 1)[e.cidx(fi, fj)];
  };
  face(r + C_FWD, i + 1, j, 1);
  face(r + C_FWD + 3, i, j + 1, 2);
  face(r + C_BWD, i, j, 1);
  face(r + C_BWD + 3, i, j, 2);
}

// the increments of the interior cells into dwi
__global__ void __launch_bounds__(256) k_impli_out(ImpliK k) {
  const Ext& e = k.e;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e.im * e.jm) return;
  const size_t q = e.cidx(1 + t % e.im, 1 + t / e.im);
#pragma unroll
  for (int v = 0; v < 5; ++v) k.dwi[q + v * e.np] = k.carry[q * K_NREC + K_DWI + v];
}

// ---------------------------------------------------------------------------
// Sweep kernel.  Per step a thread's ring entry holds its cell's record
// (C_NREC doubles), carry (K_NREC; not for a row's first cell, whose values
// are in registers) and, where the cell borders the ghost layer, the ghost
// face's flux term: a + b (i-face, first cell of a row) or a and b (j-face,
// first row).  The ghost terms depend only on the previous sweep's values of
// the boundary cells, so they are formed once per sweep, in parallel.
enum RingField { G_REC = 0, G_CARRY = 34, G_GI = 44, G_GJ = 50, G_NREC = 60 };
enum GhostTerm { T_ROW = 6, T_COL = 10 };  // doubles per row (i-face) and per column (j-face)
constexpr int kLanes = 8;          // threads per grid row in the sweep kernel (variables on 0..4)
constexpr int kMaxRowsPerCta = 64; // rows per CTA: 512 threads
constexpr int kDepth = 2;          // prefetch distance in steps
constexpr int kRing = kDepth + 1;  // entries per thread

__device__ __forceinline__ void cp16(double* dst, const double* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait_depth() { asm volatile("cp.async.wait_group %0;\n" ::"n"(kDepth - 1) : "memory"); }
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release;\n" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire;\n" ::: "memory"); }

// the cell of row j at step t of a sweep (0 if none)
__device__ __forceinline__ int step_cell(const Ext& e, int j, int t, bool fwd) {
  const int i = (fwd ? t + 2 : e.im + e.jm - t) - j;
  return (i >= 1 && i <= e.im) ? i : 0;
}

// queue thread v's share of the copies of cell (i, j)'s ring entry (the
// row's kLanes threads take the 16-byte chunks in turn)
__device__ __forceinline__ void prefetch(const ImpliK& k, double* ent, int i, int j, bool fwd, int v) {
  const Ext& e = k.e;
  const double* r = k.rec + (size_t)e.cidx(i, j) * C_NREC;
#pragma unroll
  for (int c = v; c < C_NREC / 2; c += kLanes) cp16(ent + G_REC + 2 * c, r + 2 * c);
  if (i != (fwd ? 1 : e.im)) {
    if (v < K_NREC / 2) cp16(ent + G_CARRY + 2 * v, k.carry + (size_t)e.cidx(i, j) * K_NREC + 2 * v);
  } else if (v < T_ROW / 2) {  // i-face ghost term of the row
    cp16(ent + G_GI + 2 * v, k.gterm + (size_t)(j - 1) * T_ROW + 2 * v);
  }
  if (j == (fwd ? 1 : e.jm) && v < T_COL / 2)  // j-face ghost term of the column
    cp16(ent + G_GJ + 2 * v, k.gterm + (size_t)e.jm * T_ROW + (size_t)(i - 1) * T_COL + 2 * v);
}

// F(w + dw) - F(w), G(w + dw) - G(w) of a cell from its w, f, g (at wfg) and dw
__device__ __forceinline__ void flux_delta(const ImpliK& k, const double* wfg, const double dwp[5], double df[5],
                                           double dg[5]) {
  double wi[5];
#pragma unroll
  for (int v = 0; v < 5; ++v) wi[v] = wfg[C_W + v] + dwp[v];
  const double rhom1 = __drcp_rn(wi[0]);  // correctly rounded, as 1/wi(1)
  const double velxi = wi[1] * rhom1, velyi = wi[2] * rhom1, velzi = wi[3] * rhom1;
  const double pint = k.gam1 * (wi[4] - 0.5 * wi[0] * (velxi * velxi + velyi * velyi + velzi * velzi));
  const double fi[5] = {wi[1], wi[1] * velxi + pint, wi[1] * velyi, wi[1] * velzi, velxi * (wi[4] + pint)};
  const double gi[5] = {wi[2], wi[2] * velxi, wi[2] * velyi + pint, wi[2] * velzi, velyi * (wi[4] + pint)};
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    df[v] = fi[v] - wfg[C_F + v];
    dg[v] = gi[v] - wfg[C_G + v];
  }
}

// flux term through a face (nx, ny, coef at fc) in the reference's grouping
// (lhs/impli_matrix_free.F90:186-190): a = multi (dF nx + dG ny), b = coef dw
__device__ __forceinline__ void face_term(const double* fc, const double df[5], const double dg[5],
                                          const double dwp[5], double multi, double a[5], double b[5]) {
#pragma unroll
  for (int v = 0; v < 5; ++v) {
    a[v] = multi * (df[v] * fc[0] + dg[v] * fc[1]);
    b[v] = fc[2] * dwp[v];
  }
}

// the ghost-face terms of a sweep: item b < jm is the i-face of row b+1 with
// the ghost cell (0, j) / (im+1, j), the others the j-face of column
// b-jm+1 with the ghost cell (i, 0) / (i, jm+1); the ghost's dwi is the
// previous sweep's dwi of the adjacent interior cell (read at L2: other
// threads wrote it)
__device__ __forceinline__ void ghost_terms(const ImpliK& k, bool fwd, double multi, int tid, int nthr) {
  const Ext& e = k.e;
  for (int b = tid; b < e.jm + e.im; b += nthr) {
    const bool irow = b < e.jm;
    const int i = irow ? (fwd ? 1 : e.im) : b - e.jm + 1;
    const int j = irow ? b + 1 : (fwd ? 1 : e.jm);
    const int gi = irow ? (fwd ? 0 : e.im + 1) : i, gj = irow ? j : (fwd ? 0 : e.jm + 1);
    const size_t q = e.cidx(i, j);
    double dwp[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) dwp[v] = __ldcg(k.carry + q * K_NREC + K_DWI + v);
    const double* rg = k.rec + (size_t)e.cidx(gi, gj) * C_NREC;
    double wfg[15];
#pragma unroll
    for (int v = 0; v < 15; ++v) wfg[v] = rg[v];
    double df[5], dg[5], a[5], bb[5];
    flux_delta(k, wfg, dwp, df, dg);
    // the face between the ghost and cell (i, j): that cell's bwd face (fwd
    // sweep) or fwd face (bwd sweep)
    const double* fc = k.rec + q * C_NREC + (fwd ? C_BWD : C_FWD) + (irow ? 0 : 3);
    face_term(fc, df, dg, dwp, multi, a, bb);
    if (irow) {
      double* g = k.gterm + (size_t)b * T_ROW;
#pragma unroll
      for (int v = 0; v < 5; ++v) g[v] = a[v] + bb[v];
    } else {
      double* g = k.gterm + (size_t)e.jm * T_ROW + (size_t)(i - 1) * T_COL;
#pragma unroll
      for (int v = 0; v < 5; ++v) { g[v] = a[v]; g[5 + v] = bb[v]; }
    }
  }
}

// all lmax sweeps; launched as exactly one cluster of gridDim.x CTAs of
// blockDim.x = kLanes * rb threads: the kLanes threads (r*kLanes .. r*kLanes+7)
// of CTA c own grid row j = c*rb + r + 1, thread v < 5 of a row its variable
// v+1.  A cell's update is per variable except F(w + dwi) and G(w + dwi),
// which need the cell's five w + dwi: the row's threads exchange them by warp
// shuffles (a row's threads are one 8-lane segment of a warp) and each
// variable's thread forms the pressure and velocities, then its own flux
// components, in the reference's operations.  Every thread runs the same
// sequence of cluster barrier arrives and waits (no early exit); the last
// wait follows the last shared-memory access.
__global__ void __launch_bounds__(kLanes * kMaxRowsPerCta) k_impli_sweeps(ImpliK k) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ __align__(16) double smem[];
  const Ext& e = k.e;
  const int rb = (int)blockDim.x / kLanes, rank = (int)cl.block_rank();
  const int nc = (int)gridDim.x;
  const int r = (int)threadIdx.x / kLanes, v = (int)threadIdx.x % kLanes;
  const bool var = v < 5;
  const int seg = (int)threadIdx.x & 31 & ~(kLanes - 1);  // the row's first lane in its warp
  const unsigned rowmask = 0xffu << seg;
  // the warp's threads (the last warp of a CTA may hold 8, 16 or 24)
  const int wbase = (int)threadIdx.x & ~31, nwarp = min(32, (int)blockDim.x - wbase);
  const unsigned warpmask = nwarp == 32 ? 0xffffffffu : (1u << nwarp) - 1u;
  const int j = rank * rb + r + 1;
  const bool row = j <= e.jm;
  double* slots = smem;                                                // [2][10][rb]
  double* ring = smem + (size_t)20 * ((rb + 1) / 2 * 2) + (size_t)r * kRing * G_NREC;
  auto slot = [&](double* base, int par, int c, int t) -> double* { return base + ((size_t)par * 10 + c) * rb + t; };
  double* prev_base = r > 0 ? slots : (rank > 0 ? cl.map_shared_rank(slots, rank - 1) : nullptr);
  const int prev_t = r > 0 ? r - 1 : rb - 1;
  double* next_base = r < rb - 1 ? slots : (rank < nc - 1 ? cl.map_shared_rank(slots, rank + 1) : nullptr);
  const int next_t = r < rb - 1 ? r + 1 : 0;
  const int nstep = e.im + e.jm - 1;
  const int vv = var ? v : 0;  // the variable of this thread (threads 5..7 of a row hold none)
  // carry-over of this row's last cell of the sweep (the next sweep's first)
  double last_ss = 0.0;
  // deferred store of the previous step's carry (this thread's variable)
  double* pend = nullptr;
  double pend_dw = 0.0, pend_ss = 0.0;
  const int tid = rank * (int)blockDim.x + (int)threadIdx.x, nthr = nc * (int)blockDim.x;
  cluster_arrive();  // pairs with the first wait
  for (int l = 1; l <= k.lmax; ++l) {
    const bool fwd = (l & 1) != 0;
    const double multi = 0.5 * (fwd ? 1.0 : -1.0);
    const int fo = fwd ? C_FWD : C_BWD;
    cluster_wait();  // the previous sweep's last step
    if (pend) {      // every carry of the previous sweep in memory
      pend[K_DWI + vv] = pend_dw;
      pend[K_SSOR + vv] = pend_ss;
      pend = nullptr;
    }
    cluster_arrive();
    cluster_wait();
    ghost_terms(k, fwd, multi, tid, nthr);
    cluster_arrive();
    cluster_wait();
    // prologue: the entries of steps 0 .. kDepth-1
#pragma unroll
    for (int t = 0; t < kDepth; ++t) {
      const int i = row ? step_cell(e, j, t, fwd) : 0;
      if (i) prefetch(k, ring + (t % kRing) * G_NREC, i, j, fwd, v);
      cp_commit();
    }
    double ci = 0.0;  // a + b of the i-face term of this row's next cell (this thread's variable)
    for (int t = 0; t < nstep; ++t) {
      const int par = t & 1;
      const int i = row ? step_cell(e, j, t, fwd) : 0;
      cp_wait_depth();  // this thread's copies of this step's entry have landed
      __syncwarp(warpmask);  // and the other seven threads' copies of the row's entry
      if (t > 0) cluster_wait();  // the neighbouring rows' slots of step t-1 are written
      if (i) {  // the same for the row's kLanes threads
        const double* ent = ring + (t % kRing) * G_NREC;
        const double* rr = ent + G_REC;
        const bool first = i == (fwd ? 1 : e.im);
        // the update (lhs/impli_matrix_free.F90:199-222) of this thread's variable
        double ssn = 0.0, dwn = 0.0, wv = 0.0;
        if (var) {
          const double sso = first ? last_ss : ent[G_CARRY + K_SSOR + v];
          if (first) ci = ent[G_GI + v];  // i-face term from the ghost cell
          double aj, bj;
          if (j == (fwd ? 1 : e.jm)) {  // j-face term from the ghost row
            aj = ent[G_GJ + v];
            bj = ent[G_GJ + 5 + v];
          } else {
            const double* nb = fwd ? prev_base : next_base;
            const int nt = fwd ? prev_t : next_t;
            aj = *slot(const_cast<double*>(nb), par ^ 1, v, nt);
            bj = *slot(const_cast<double*>(nb), par ^ 1, 5 + v, nt);
          }
          ssn = ((ci + aj) + bj) * rr[C_TAU0];
          dwn = (ssn + (rr[C_D1W + v] + sso)) * rr[C_CDM1];
          wv = rr[C_W + v] + dwn;
        }
        // the cell's w + dwi on every thread of the row
        double wi[5];
#pragma unroll
        for (int m = 0; m < 5; ++m) wi[m] = __shfl_sync(rowmask, wv, seg + m);
        if (var) {
          // this variable of F(w + dwi) - F(w), G(w + dwi) - G(w)
          const double rhom1 = __drcp_rn(wi[0]);  // correctly rounded, as 1/wi(1)
          const double velxi = wi[1] * rhom1, velyi = wi[2] * rhom1, velzi = wi[3] * rhom1;
          const double pint = k.gam1 * (wi[4] - 0.5 * wi[0] * (velxi * velxi + velyi * velyi + velzi * velzi));
          const double hp = wi[4] + pint;
          // fi = (wi2, wi2 u + p, wi2 v, wi2 w, u (wi5 + p)), gi = (wi3, wi3 u, wi3 v + p, wi3 w, v (wi5 + p))
          const double fa = v == 4 ? hp : wi[1], ga = v == 4 ? hp : wi[2];
          const double fm = v == 0 ? 1.0 : (v == 1 || v == 4) ? velxi : v == 2 ? velyi : velzi;
          const double gm = v == 0 ? 1.0 : v == 1 ? velxi : (v == 2 || v == 4) ? velyi : velzi;
          const double fi = fa * fm + (v == 1 ? pint : 0.0), gi = ga * gm + (v == 2 ? pint : 0.0);
          const double df = fi - rr[C_F + v], dg = gi - rr[C_G + v];
          // this cell's terms for its downstream faces
          // (lhs/impli_matrix_free.F90:186-190): a = multi (dF nx + dG ny), b = coef dw
          if (fwd ? j < e.jm : j > 1) {
            const double* fc = rr + fo + 3;
            *slot(slots, par, v, r) = multi * (df * fc[0] + dg * fc[1]);
            *slot(slots, par, 5 + v, r) = fc[2] * dwn;
          }
          if (fwd ? i < e.im : i > 1) {
            const double* fc = rr + fo;
            ci = multi * (df * fc[0] + dg * fc[1]) + fc[2] * dwn;
          } else {  // the row's last cell of this sweep: the next sweep's first
            last_ss = ssn;
          }
        }
        cluster_arrive();
        if (pend) {
          pend[K_DWI + vv] = pend_dw;
          pend[K_SSOR + vv] = pend_ss;
        }
        pend = var ? k.carry + (size_t)e.cidx(i, j) * K_NREC : nullptr;
        pend_dw = dwn;
        pend_ss = ssn;
      } else {
        cluster_arrive();
      }
      // the entry of step t + kDepth
      const int in = (row && t + kDepth < nstep) ? step_cell(e, j, t + kDepth, fwd) : 0;
      if (in) prefetch(k, ring + ((t + kDepth) % kRing) * G_NREC, in, j, fwd, v);
      cp_commit();
    }
  }
  if (pend) {
    pend[K_DWI + vv] = pend_dw;
    pend[K_SSOR + vv] = pend_ss;
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  cluster_wait();  // pairs with the last arrive; no CTA leaves while its slots may be read
}


// slots (2 parities x 10 values per row, padded to 16 bytes) and the rings
size_t sweep_smem(int rb) { return ((size_t)20 * ((rb + 1) / 2 * 2) + (size_t)rb * kRing * G_NREC) * sizeof(double); }

// chosen cluster size per device (the function attributes are set for the
// device current at the first call there)
constexpr int kMaxDev = 64;
int g_cluster[kMaxDev] = {0};
std::mutex g_cluster_mu;

int pick_cluster() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) { cudaGetLastError(); return 8; }
  std::lock_guard<std::mutex> lk(g_cluster_mu);
  if (g_cluster[dev]) return g_cluster[dev];
  int nc = 8;
  cudaFuncSetAttribute(k_impli_sweeps, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_smem(kMaxRowsPerCta));
  if (cudaFuncSetAttribute(k_impli_sweeps, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(16);
    cfg.blockDim = dim3(kMaxRowsPerCta * kLanes);
    cfg.dynamicSmemBytes = sweep_smem(kMaxRowsPerCta);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 16;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nclusters = 0;
    if (cudaOccupancyMaxActiveClusters(&nclusters, k_impli_sweeps, &cfg) == cudaSuccess && nclusters >= 1) nc = 16;
  }
  cudaGetLastError();  // a refused query leaves the portable size
  g_cluster[dev] = nc;
  return nc;
}

}  // namespace

size_t impli_scratch_doubles(int im, int jm, int gh) {
  const size_t np = (size_t)(im + 2 * gh) * (size_t)(jm + 2 * gh);
  return np * (C_NREC + K_NREC + I_NPLANE) + (size_t)T_ROW * jm + (size_t)T_COL * im + 2;  // + 2: 16-byte alignment
}

int impli_cluster_size() { return pick_cluster(); }

int impli_max_rows() { return kMaxRowsPerCta * pick_cluster(); }

cudaError_t run_impli(const ImpliArgs& a, cudaStream_t st) {
  ImpliK k;
  k.e = make_ext(a.im, a.jm, a.gh);
  k.lmax = a.lmax;
  k.dtcoef = a.dtcoef; k.cfl = a.cfl; k.gam = a.gam; k.rgaz = a.rgaz;
  k.gampr = 2.0 * a.gam / a.prandtl;
  k.gam1 = a.gam - 1.0;
  k.cvm1 = 1.0 / a.cv;
  k.betas = a.muref * (a.tref + a.cs) / (sqrt(a.tref) * a.tref);
  k.s_suth = a.s_suth;
  k.nx = a.nx; k.ny = a.ny; k.w = a.w; k.dw = a.dw; k.vol = a.vol; k.volf = a.volf;
  k.dwi = a.dwi;
  // records first, 16-byte aligned (the 16-byte copies need it)
  double* base = a.scratch + ((reinterpret_cast<uintptr_t>(a.scratch) & 15) ? 1 : 0);
  const size_t np = k.e.np;
  k.rec = base;
  k.carry = base + np * C_NREC;
  k.gterm = k.carry + np * K_NREC;
  k.sc = k.gterm + (size_t)T_ROW * a.jm + (size_t)T_COL * a.im;
  const int nc = pick_cluster();
  const int rb = (a.jm + nc - 1) / nc;  // rows per CTA
  if (a.lmax >= 1 && rb > kMaxRowsPerCta) return cudaErrorInvalidValue;
  const int B = 256;
  const unsigned gc = (unsigned)((np + B - 1) / B), gi = (unsigned)((a.im * a.jm + B - 1) / B);
  k_impli_cells<<<gc, B, 0, st>>>(k);
  k_impli_faces<<<gc, B, 0, st>>>(k);
  k_impli_diag<<<gi, B, 0, st>>>(k);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess || a.lmax < 1) return err;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)nc);
  cfg.blockDim = dim3((unsigned)(rb * kLanes));
  cfg.dynamicSmemBytes = sweep_smem(rb);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)nc;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  err = cudaLaunchKernelEx(&cfg, k_impli_sweeps, k);
  if (err != cudaSuccess) return err;
  k_impli_out<<<gi, B, 0, st>>>(k);
  return cudaGetLastError();
}

}  // namespace bcg
