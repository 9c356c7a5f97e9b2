/* broadcast_gb300.h - C ABI of libbroadcast_gb300.so, the GB300 (sm_103a)
 * implementation of BROADCAST's DNC5 residual / tangent / boundary /
 * colored-Jacobian hot path.
 *
 * Each entry point replaces one f2py-wrapped Fortran routine of the reference
 * and keeps its name (prefixed bcg_) and argument order; the reference routine
 * it replaces is cited on each declaration.  Conventions:
 *
 *  - Arrays are double precision, Fortran (column-major) order, with the
 *    caller's ghost-padded extents: cell arrays (im+2gh, jm+2gh[, nv]), face
 *    and node arrays (im+2gh+1, jm+2gh+1[, 2]).  Outputs are written in place,
 *    as with the reference's intent(inout) arguments.
 *  - An array may be a host pointer or a CUDA device pointer.  Host arrays
 *    are copied to the device and back around the call, which has completed
 *    when it returns.  When every array is a device pointer the work is queued
 *    on the library stream (bcg_set_stream) and the call returns at once.
 *  - interf/prr/prd are the reference's Fortran (2,2) integer arrays in
 *    column-major order {imin, imax, jmin, jmax}; loc is one of "Ilo", "Ihi",
 *    "Jlo", "Jhi" (3 characters, no terminator needed).  These small index
 *    arrays are always host pointers.
 *  - Every function returns 0 on success or a negative code: -1 bad arguments,
 *    -2 CUDA failure, -3 device allocation failure, -4 no CUDA device, -5 a
 *    singular matrix in the linear solve.
 *    bcg_last_error_string() describes the last failure of the calling thread.
 *  - Trailing dimension arguments that f2py infers from array shapes (lm, em,
 *    nbentry) are explicit here.
 *  - Calls are serialised on one library stream per process; two host threads
 *    must not call the library at the same time.
 */
#ifndef BROADCAST_GB300_H
#define BROADCAST_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- runtime --------------------------------------------------------------- */
int bcg_abi_version(void);
int bcg_set_stream(void* cuda_stream);      /* NULL selects the legacy default stream */
void* bcg_get_stream(void);
int bcg_synchronize(void);
const char* bcg_last_error_string(void);
size_t bcg_residual_scratch_bytes(int im, int jm, int gh, int ndir);

/* ---- residual, tangent ------------------------------------------------------ */
/* srcfv/rhs/flux_num_dnc5.F90:7-8 (flux_num_dnc5_2d).  x0, y0, xc, yc are
 * accepted for signature compatibility and unused, as in the reference. */
int bcg_flux_num_dnc5_2d(double* residu, const double* w, const double* x0, const double* y0, const double* nx,
                         const double* ny, const double* xc, const double* yc, const double* vol, const double* volf,
                         int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs,
                         double muref, double tref, double s_suth, double k2, double k4, int im, int jm);

/* srcfv/tangent/flux_num_dnc5_d.f90:15-17 (FLUX_NUM_DNC5_2D_D): residu and
 * residud = dR/dw . wd */
int bcg_flux_num_dnc5_2d_d(double* residu, double* residud, const double* w, const double* wd, const double* x0,
                           const double* y0, const double* nx, const double* ny, const double* xc, const double* yc,
                           const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                           double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
                           double k4, int im, int jm);

/* Batched form of FLUX_NUM_DNC5_2D_D (no reference counterpart beyond the
 * routine it batches): nd tangent states stacked in wd, nd outputs in residud,
 * one primal evaluation per group of up to 4 directions. */
int bcg_flux_num_dnc5_2d_dn(double* residu, double* residud, const double* w, const double* wd, int nd,
                            const double* x0, const double* y0, const double* nx, const double* ny, const double* xc,
                            const double* yc, const double* vol, const double* volf, int gh, double cp, double cv,
                            double prandtl, double gam, double rgaz, double cs, double muref, double tref,
                            double s_suth, double k2, double k4, int im, int jm);

/* srcfv/rhs/flux_num_dnc5_nowall.F90:7 flux_num_dnc5_nowall_2d and its tangent
 * srcfv/tangent/flux_num_dnc5_nowall_d.f90 flux_num_dnc5_nowall_2d_d: the same
 * scheme with the centred fluxes on every row j = 1..jm+1 (no near-wall rows,
 * no wall face); same arguments as flux_num_dnc5_2d / _d. */
int bcg_flux_num_dnc5_nowall_2d(double* residu, const double* w, const double* x0, const double* y0,
                                const double* nx, const double* ny, const double* xc, const double* yc,
                                const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                                double gam, double rgaz, double cs, double muref, double tref, double s_suth,
                                double k2, double k4, int im, int jm);
int bcg_flux_num_dnc5_nowall_2d_d(double* residu, double* residud, const double* w, const double* wd,
                                  const double* x0, const double* y0, const double* nx, const double* ny,
                                  const double* xc, const double* yc, const double* vol, const double* volf, int gh,
                                  double cp, double cv, double prandtl, double gam, double rgaz, double cs,
                                  double muref, double tref, double s_suth, double k2, double k4, int im, int jm);

/* srcfv/adjoint/flux_num_dnc5_nowall_b.f90: the adjoint of flux_num_dnc5_nowall_2d,
 * with the arguments of flux_num_dnc5_2d_b. */
int bcg_flux_num_dnc5_nowall_2d_b(double* residu, double* residub, const double* w, double* wb, const double* x0,
                                  const double* y0, const double* nx, const double* ny, const double* xc,
                                  const double* yc, const double* vol, const double* volf, int gh, double cp,
                                  double cv, double prandtl, double gam, double rgaz, double cs, double muref,
                                  double tref, double s_suth, double k2, double k4, int im, int jm);

/* The schemes of order 3, 7 and 9 and their tangents, with the arguments of
 * flux_num_dnc5_2d / _d (gh >= (order+1)/2; im, jm >= 6, and >= 9 for DNC7 and
 * >= 11 for DNC9, whose wall rows read that many cell rows):
 *   srcfv/rhs/flux_num_dnc3.F90:7, flux_num_dnc7.F90:7, flux_num_dnc9.F90:7
 *   srcfv/rhs/flux_num_dnc{3,7,9}_nowall.F90:7
 *   srcfv/tangent/flux_num_dnc{3,7,9}_d.f90, flux_num_dnc{3,7,9}_nowall_d.f90 */
int bcg_flux_num_dnc3_2d(double* residu, const double* w, const double* x0, const double* y0, const double* nx,
    const double* ny, const double* xc, const double* yc, const double* vol, const double* volf, int gh, double cp,
    double cv, double prandtl, double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
    double k4, int im, int jm);
int bcg_flux_num_dnc3_2d_d(double* residu, double* residud, const double* w, const double* wd, const double* x0,
    const double* y0, const double* nx, const double* ny, const double* xc, const double* yc, const double* vol,
    const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs, double muref,
    double tref, double s_suth, double k2, double k4, int im, int jm);
int bcg_flux_num_dnc3_nowall_2d(double* residu, const double* w, const double* x0, const double* y0, const double* nx,
    const double* ny, const double* xc, const double* yc, const double* vol, const double* volf, int gh, double cp,
    double cv, double prandtl, double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
    double k4, int im, int jm);
int bcg_flux_num_dnc3_nowall_2d_d(double* residu, double* residud, const double* w, const double* wd, const double* x0,
    const double* y0, const double* nx, const double* ny, const double* xc, const double* yc, const double* vol,
    const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs, double muref,
    double tref, double s_suth, double k2, double k4, int im, int jm);
int bcg_flux_num_dnc7_2d(double* residu, const double* w, const double* x0, const double* y0, const double* nx,
    const double* ny, const double* xc, const double* yc, const double* vol, const double* volf, int gh, double cp,
    double cv, double prandtl, double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
    double k4, int im, int jm);
int bcg_flux_num_dnc7_2d_d(double* residu, double* residud, const double* w, const double* wd, const double* x0,
    const double* y0, const double* nx, const double* ny, const double* xc, const double* yc, const double* vol,
    const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs, double muref,
    double tref, double s_suth, double k2, double k4, int im, int jm);
int bcg_flux_num_dnc7_nowall_2d(double* residu, const double* w, const double* x0, const double* y0, const double* nx,
    const double* ny, const double* xc, const double* yc, const double* vol, const double* volf, int gh, double cp,
    double cv, double prandtl, double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
    double k4, int im, int jm);
int bcg_flux_num_dnc7_nowall_2d_d(double* residu, double* residud, const double* w, const double* wd, const double* x0,
    const double* y0, const double* nx, const double* ny, const double* xc, const double* yc, const double* vol,
    const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs, double muref,
    double tref, double s_suth, double k2, double k4, int im, int jm);
int bcg_flux_num_dnc9_2d(double* residu, const double* w, const double* x0, const double* y0, const double* nx,
    const double* ny, const double* xc, const double* yc, const double* vol, const double* volf, int gh, double cp,
    double cv, double prandtl, double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
    double k4, int im, int jm);
int bcg_flux_num_dnc9_2d_d(double* residu, double* residud, const double* w, const double* wd, const double* x0,
    const double* y0, const double* nx, const double* ny, const double* xc, const double* yc, const double* vol,
    const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs, double muref,
    double tref, double s_suth, double k2, double k4, int im, int jm);
int bcg_flux_num_dnc9_nowall_2d(double* residu, const double* w, const double* x0, const double* y0, const double* nx,
    const double* ny, const double* xc, const double* yc, const double* vol, const double* volf, int gh, double cp,
    double cv, double prandtl, double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
    double k4, int im, int jm);
int bcg_flux_num_dnc9_nowall_2d_d(double* residu, double* residud, const double* w, const double* wd, const double* x0,
    const double* y0, const double* nx, const double* ny, const double* xc, const double* yc, const double* vol,
    const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz, double cs, double muref,
    double tref, double s_suth, double k2, double k4, int im, int jm);

/* The linear solve of the SER Newton iteration (BROADCAST_npz.py:1146-1158,
 * where the reference factorises J with PETSc/MUMPS, misc/PETSc_func.py:137-152):
 * x = A^-1 b for the n x n CSR matrix A (int32 indptr[n+1] and indices[nnz],
 * double data[nnz]; duplicates summed) by band LU with partial pivoting on the
 * GPU (LAPACK's blocked dgbtrf/dgbtrs algorithm through cuSOLVER getrf panels
 * and cuBLAS trsm/gemm on views of the band storage, which takes
 * 8 n (3 kl + ku + 2 nb + 1) bytes of device memory for bandwidths kl, ku).
 * perm (optional, may be null): row and column k of A are row and column perm[k]
 * of the factorised matrix, a bandwidth-reducing order (e.g. the folded
 * azimuthal order of a periodic O-mesh); must be a permutation of 0..n-1.
 * nb: block size (0: 256).  Returns -5 with *info = the first zero pivot
 * (1-based) for a singular matrix.  No reference counterpart in f2py: the
 * reference calls PETSc here. */
int bcg_csr_band_lu_solve(int n, const int* indptr, const int* indices, const double* data, long long nnz,
                          const int* perm, const double* b, double* x, int nb, int* info);

/* srcfv/lhs/impli_matrix_free.F90:7 (IMPLI_MATRIX_FREE_2D): the implicit phase
 * of the 'impli' time marching (BROADCAST_npz.py:911-941): lmax symmetric
 * Gauss-Seidel sweeps of the scalar-diagonal implicit operator on the
 * right-hand side dw (the residual); dwi is overwritten with the increment
 * (every ghost zero).  em must be 5.  The sweeps run as one launch of one
 * thread-block cluster (anti-diagonal wavefront, cluster barrier per diagonal). */
int bcg_impli_matrix_free_2d(double* dwi, const double* nx, const double* ny, const double* w, const double* dw,
                             const double* vol, const double* volf, double dtcoef, double cfl, double gam, double rgaz,
                             double prandtl, int lmax, int gh, double cv, double cs, double muref, double tref,
                             double s_suth, int im, int jm, int em);

/* srcfv/adjoint/flux_num_dnc5_b.f90:15 (FLUX_NUM_DNC5_2D_B): wb = (dR/dw)^T residub
 * on every padded cell (wb overwritten); the interior of residub is zeroed on
 * return, as in the reference; residu is unused. */
int bcg_flux_num_dnc5_2d_b(double* residu, double* residub, const double* w, double* wb, const double* x0,
                           const double* y0, const double* nx, const double* ny, const double* xc, const double* yc,
                           const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                           double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
                           double k4, int im, int jm);
/* nd cotangents at once (no reference counterpart; the drivers loop over
 * flux_num_dnc5_2d_b, cylinder.py:1116-1159): residub and wb hold nd
 * consecutive (ni, nj, 5) blocks; same result as nd calls of
 * bcg_flux_num_dnc5_2d_b, bit for bit. */
int bcg_flux_num_dnc5_2d_bn(double* residu, double* residub, const double* w, double* wb, int nd, const double* x0,
                            const double* y0, const double* nx, const double* ny, const double* xc, const double* yc,
                            const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                            double gam, double rgaz, double cs, double muref, double tref, double s_suth, double k2,
                            double k4, int im, int jm);

/* ---- boundary conditions ---------------------------------------------------- */
/* srcfv/borders/bc_wall_viscous.F90:2 ; tangent/bc_wall_viscous_d.f90:11 */
int bcg_bc_wall_viscous_adia_2d(double* w, const char* loc, double gam, const int* interf, int gh, int im, int jm);
int bcg_bc_wall_viscous_adia_2d_d(double* w, double* wd, const char* loc, double gam, const int* interf, int gh,
                                  int im, int jm);
/* srcfv/borders/bc_no_reflexion.F90:8 ; tangent/bc_no_reflexion_d.f90:16 (wbd is (lm,5)) */
int bcg_bc_no_reflexion_2d(double* w, const double* wbd, const char* loc, const int* interf, const double* nx,
                           const double* ny, double gam, int gh, int im, int jm, int lm);
int bcg_bc_no_reflexion_2d_d(double* w, double* wd, const double* wbd, const char* loc, const int* interf,
                             const double* nx, const double* ny, double gam, int gh, int im, int jm, int lm);
/* srcfv/borders/bc_supandsubinlet.F90:2 ; tangent/bc_supandsubinlet_d.f90:11 (field is (lm,gh,5)) */
int bcg_bc_supandsubinlet_2d(double* w, const char* loc, const int* interf, const double* field, const double* nx,
                             const double* ny, double gam, int im, int jm, int lm, int gh);
int bcg_bc_supandsubinlet_2d_d(double* w, double* wd, const char* loc, const int* interf, const double* field,
                               const double* nx, const double* ny, double gam, int im, int jm, int lm, int gh);
/* srcfv/borders/bc_extrapolate.F90:39 ; tangent/bc_extrapolateo2_d.f90:18 (em variables) */
int bcg_bc_extrapolate_o2_2d(double* w, const char* loc, const int* interf, int im, int jm, int gh, int em);
int bcg_bc_extrapolate_o2_2d_d(double* w, double* wd, const char* loc, const int* interf, int im, int jm, int gh,
                               int em);
/* srcfv/borders/jn_match.F90:3 ; tangent/jn_match_2d_d.f90:11 */
int bcg_jn_match_2d(double* wr, const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr, int jmr,
                    const double* wd, const int* prd, int gh1d, int gh2d, int gh3d, int gh4d, int imd, int jmd,
                    const int* tr, int em);
int bcg_jn_match_2d_d(double* wr, double* wrd, const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr,
                      int jmr, const double* wd, const double* wdd, const int* prd, int gh1d, int gh2d, int gh3d,
                      int gh4d, int imd, int jmd, const int* tr, int em);
/* ---- adjoints of the fills (srcfv/adjoint, module f_adj) ---------------------- */
/* bc_wall_viscous_b.f90:11, bc_no_reflexion_b.f90:16, bc_supandsubinlet_b.f90:11,
 * bc_extrapolateo2_b.f90:18: wb(cells the fill reads) += J^T wb(ghosts), then
 * wb(written ghosts) = 0; w (the state before the fill) is left unchanged.
 * jn_match_2d_b.f90:1: wdb = 0 over its whole extent, then wdb(donor) +=
 * wrb(receiver) and wrb(receiver) = 0; wr and wd are not read. */
int bcg_bc_wall_viscous_adia_2d_b(double* w, double* wb, const char* loc, double gam, const int* interf, int gh,
                                  int im, int jm);
int bcg_bc_no_reflexion_2d_b(double* w, double* wb, const double* wbd, const char* loc, const int* interf,
                             const double* nx, const double* ny, double gam, int gh, int im, int jm, int lm);
int bcg_bc_supandsubinlet_2d_b(double* w, double* wb, const char* loc, const int* interf, const double* field,
                               const double* nx, const double* ny, double gam, int im, int jm, int lm, int gh);
int bcg_bc_extrapolate_o2_2d_b(double* w, double* wb, const char* loc, const int* interf, int im, int jm, int gh,
                               int em);
int bcg_jn_match_2d_b(double* wr, double* wrb, const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr,
                      int jmr, const double* wd, double* wdb, const int* prd, int gh1d, int gh2d, int gh3d, int gh4d,
                      int imd, int jmd, const int* tr, int em);

/* srcfv/borders/jn_match_geom.F90:7 (tr(1) = +-1 only) */
int bcg_jn_match_geom_2d(double* wr, const int* prr, int gh1r, int gh2r, int gh3r, int gh4r, int imr, int jmr,
                         const double* wd, const int* prd, int gh1d, int gh2d, int gh3d, int gh4d, int imd, int jmd,
                         const int* tr);

/* ---- colored Jacobian assembly (misc/ComputeJacobian.f90) -------------------- */
/* :357 testvector ; :1075 testvector_partial */
int bcg_testvector(double* wd, int m, int l, int k, int gh, int im, int jm);
int bcg_testvector_partial(double* wd, int m, int l, int k, int gh, int im, int jm, int istart, int iend, int jstart,
                           int jend);
/* :292 computejacobianfromjv ; :503 _relaxed ; :847 _relaxed_withjn ; :929 _withjn ;
 * :1095 _relaxed_withjnandcheck ; :708 computejacobianfromdz.  jac/ia/ja hold
 * nbentry entries; only the 5*im*jm slots of the given seed are written. */
int bcg_computejacobianfromjv(double* jac, int* ia, int* ja, const double* resd, int m, int l, int k, int gh, int im,
                              int jm, long long nbentry);
int bcg_computejacobianfromjv_relaxed(double* jac, int* ia, int* ja, const double* resd, int m, int l, int k, int gh,
                                      int im, int jm, long long nbentry, const double* coefdiag);
int bcg_computejacobianfromjv_relaxed_withjn(double* jac, int* ia, int* ja, const double* resd, int m, int l, int k,
                                             int gh, int im, int jm, long long nbentry, const double* coefdiag);
int bcg_computejacobianfromjv_withjn(double* jac, int* ia, int* ja, const double* resd, int m, int l, int k, int gh,
                                     int im, int jm, long long nbentry);
int bcg_computejacobianfromjv_relaxed_withjnandcheck(double* jac, int* ia, int* ja, const double* resd, int m, int l,
                                                     int k, int gh, int im, int jm, long long nbentry,
                                                     const double* coefdiag, double mini, int n);
int bcg_computejacobianfromdz(double* jac, int* ia, int* ja, const double* dz, int m, int l, int k, int gh, int im,
                              int jm, long long nbentry);

/* Batched assembly of the boundary-layer configuration's Jacobian, all 245
 * colour seeds in one call, as CSR (the loop of BROADCAST_npz.py:1068-1137:
 * testvector, the linearised boundary chain inlet Ilo / no-reflexion Jhi /
 * extrapolation Ihi / wall Jlo, flux_num_dnc5_2d_d, computejacobianfromjv
 * [_relaxed when coefdiag is not NULL], remove_zero_jac keeping |a| > mini; the
 * COO -> CSR of misc/PETSc_func.py:71-96; with divide_by_vol, the Jacvol scaling
 * of BROADCAST_npz.py:1206-1210).  w must hold the primal boundary fills.  Rows
 * are 5*im*jm, columns sorted within a row; *nnz receives the entry count (also
 * when capacity is too small, which returns -1). */
int bcg_jacobian_dnc5_bl_csr(const double* w, const double* nx, const double* ny, const double* vol,
                             const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz,
                             double cs, double muref, double tref, double s_suth, double k2, double k4, int im, int jm,
                             const int* interf_ilo, const int* interf_jhi, const int* interf_ihi,
                             const int* interf_jlo, const double* field, int lm_field, const double* wbd, int lm_wbd,
                             const double* coefdiag, double mini, int divide_by_vol, int* indptr, int* indices,
                             double* data, long long capacity, long long* nnz);

/* Same for the periodic O-mesh of cylinder.py:900-980: the tangent boundary
 * chain of handleBC.applyBC (no-reflexion Jhi, wall Jlo, the joins prr1 <- prd2
 * and prr2 <- prd1 twice, as jn_match_2d_d), flux_num_dnc5_2d_d and
 * computejacobianfromjv[_relaxed]_withjn, whose columns wrap periodically in
 * i.  When im is not a multiple of 7 the seeds of one colour would meet
 * within a stencil across the periodic join, so, as the driver does
 * (cylinder.py:899-938), the seeds run in two azimuthal zones (columns below
 * and from im/2/7*7, testvector_partial, 490 seeds) with the columns of
 * computejacobianfromjv_relaxed_withjnandcheck; slots that land on one
 * column are summed, as the COO -> CSR conversion does. */
int bcg_jacobian_dnc5_cyl_csr(const double* w, const double* nx, const double* ny, const double* vol,
                              const double* volf, int gh, double cp, double cv, double prandtl, double gam,
                              double rgaz, double cs, double muref, double tref, double s_suth, double k2, double k4,
                              int im, int jm, const int* interf_jhi, const int* interf_jlo, const double* wbd,
                              int lm_wbd, const int* prr1, const int* prd1, const int* prr2, const int* prd2,
                              const int* tr, const double* coefdiag, double mini, int divide_by_vol, int* indptr,
                              int* indices, double* data, long long capacity, long long* nnz);

/* Same loop for the spanwise operators (BROADCAST_npz.py:1221-1249): per seed,
 * testvector, the same linearised boundary chain, coeffs_5p_dz (which = 1) or
 * coeffs_5p_dz2 (which = 2), computejacobianfromdz (+dz, its own row window),
 * remove_zero_jac with mini; then CSR as above (no volume scaling). */
int bcg_jacobian_dz_bl_csr(const double* w, const double* nx, const double* ny, const double* vol,
                           const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz,
                           double cs, double muref, double tref, double s_suth, int im, int jm, const int* interf_ilo,
                           const int* interf_jhi, const int* interf_ihi, const int* interf_jlo, const double* field,
                           int lm_field, const double* wbd, int lm_wbd, int which, double mini, int* indptr,
                           int* indices, double* data, long long capacity, long long* nnz);

/* Global-stability operator J(beta) = J - beta^2 Dzz + i beta Dz (biglobal.py:82,
 * where PETSc adds the three matrices on the union of their patterns) for
 * nbeta wavenumbers at once: CSR inputs of nrow rows with sorted columns (the
 * outputs of the two calls above); indptr/indices receive the union pattern,
 * values nbeta planes of *nnz complex numbers (re, im interleaved; plane k at
 * values + 2*k*(*nnz)).  Returns -1 with *nnz set when capacity is too small. */
int bcg_csr_spanwise_beta(int nrow, const int* j_indptr, const int* j_indices, const double* j_data,
                          const int* dz_indptr, const int* dz_indices, const double* dz_data, const int* dzz_indptr,
                          const int* dzz_indices, const double* dzz_data, int nbeta, const double* betas, int* indptr,
                          int* indices, double* values, long long capacity, long long* nnz);

/* ---- spanwise operators (srcfv/dz, module f_dz) -------------------------------- */
/* coeffs_5p_dz.F90:10 coeffs_5p_dz : dz_out = Dz . wd (coefficient of i*beta)
 * coeffs_5p_dz2.F90:10 coeffs_5p_dz2: dz2_out = Dzz . wd (coefficient of -beta^2)
 * Interior of the output written, ghosts untouched; x0, y0, xc, yc, volf unused
 * (as in the reference), nx, ny, vol unused by coeffs_5p_dz2. */
int bcg_coeffs_5p_dz(double* dz_out, const double* w, const double* wd, const double* x0, const double* y0,
                     const double* nx, const double* ny, const double* xc, const double* yc, const double* vol,
                     const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz,
                     double cs, double muref, double tref, double s_suth, int im, int jm);
int bcg_coeffs_5p_dz2(double* dz2_out, const double* w, const double* wd, const double* x0, const double* y0,
                      const double* nx, const double* ny, const double* xc, const double* yc, const double* vol,
                      const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz,
                      double cs, double muref, double tref, double s_suth, int im, int jm);
/* nd directions at once (wd and the output hold nd stacked padded arrays);
 * no reference counterpart, equivalent to nd calls of the routines above. */
int bcg_coeffs_5p_dz_dn(double* dz_out, const double* w, const double* wd, int nd, const double* x0,
                        const double* y0, const double* nx, const double* ny, const double* xc, const double* yc,
                        const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                        double gam, double rgaz, double cs, double muref, double tref, double s_suth, int im, int jm);
int bcg_coeffs_5p_dz2_dn(double* dz2_out, const double* w, const double* wd, int nd, const double* x0,
                         const double* y0, const double* nx, const double* ny, const double* xc, const double* yc,
                         const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                         double gam, double rgaz, double cs, double muref, double tref, double s_suth, int im,
                         int jm);

/* ---- norms (srcfv/norm.F90) ---------------------------------------------------- */
/* :2 compute_norml2 ; :34 compute_norml2inf ; :79 compute_maxnorm (5-vectors) */
int bcg_compute_norml2(double* norm, double* nmoy, const double* rhs, int im, int jm, int gh);
int bcg_compute_norml2inf(double* norm, double* ninf, const double* rhs, int im, int jm, int gh);
int bcg_compute_maxnorm(double* norm, int* imax, int* jmax, const double* rhs, int im, int jm, int gh);

/* ---- one-time pre-processing (host) ------------------------------------------- */
/* srcfv/geom/computegeom.F90:3 */
int bcg_computegeom_2d(double* x0, double* y0, double* nx, double* ny, double* xc, double* yc, double* vol,
                       double* volf, int im, int jm, int gh);
/* set_bnd.f90:1 (field is (jm,gh,5), wbd is (im+gh,5)) */
int bcg_set_bndbl_2d(const double* w, double* field, double* wbd, int im, int jm, int gh);
/* initialisation.f90:2 */
int bcg_initblfv(double muinf, const double* xc, const double* yc, double* w, double* field, int im, int gh, int jm);

/* J (J/vol with divide_by_vol = 1), Dz and Dzz of the boundary layer from ONE
 * pass over the 245 seeds (BROADCAST_npz.py:1068-1137 and 1221-1249: the same
 * testvector and linearised boundary chain feed flux_num_dnc5_2d_d,
 * coeffs_5p_dz and coeffs_5p_dz2), each filtered by |a| > mini into its CSR
 * (computejacobianfromjv, computejacobianfromdz), then, with nbeta > 0, J(beta)
 * = J - beta^2 Dzz + i beta Dz for the host list betas as the epilogue (as
 * bcg_csr_spanwise_beta).  The three CSR outputs are device arrays given by
 * tables of three device addresses (J, Dz, Dzz); capacity3 and nnz3 hold three
 * counts each; the J(beta) outputs are device arrays too. */
int bcg_jacobian_span_bl_csr(const double* w, const double* nx, const double* ny, const double* vol,
                             const double* volf, int gh, double cp, double cv, double prandtl, double gam, double rgaz,
                             double cs, double muref, double tref, double s_suth, double k2, double k4, int im, int jm,
                             const int* interf_ilo, const int* interf_jhi, const int* interf_ihi,
                             const int* interf_jlo, const double* field, int lm_field, const double* wbd, int lm_wbd,
                             double mini, int divide_by_vol, const unsigned long long* indptr3,
                             const unsigned long long* indices3, const unsigned long long* data3,
                             const long long* capacity3, long long* nnz3, int nbeta, const double* betas,
                             int* b_indptr, int* b_indices, double* b_values, long long b_capacity, long long* b_nnz);

/* ---- uneven batch of grids (no counterpart in the reference, which runs one
 * grid per process) ---------------------------------------------------------- */
/* A plan for ngrid independent grids (gh = 3, im, jm >= 6 each; phys holds the
 * 11 scalars cp cv prandtl gam rgaz cs muref tref s_suth k2 k4 of each grid)
 * computing the residual (ndir = 0) or the residual and one tangent direction
 * (ndir = 1) of every grid: each pass of the DNC5 residual is one persistent
 * launch over the tiles of all grids.  The plan owns its device scratch
 * (bcg_batch_device_bytes) until bcg_batch_destroy. */
int bcg_batch_create(int ngrid, const int* im, const int* jm, const double* phys, int ndir, long long* plan);
/* Device addresses of each grid's arrays (host tables of ngrid entries): w, wd
 * (one padded direction), nx, ny, vol, volf, residu, residud (interior
 * written).  May be called again between runs; a captured graph stays valid. */
int bcg_batch_set_arrays(long long plan, const unsigned long long* w, const unsigned long long* wd,
                         const unsigned long long* nx, const unsigned long long* ny, const unsigned long long* vol,
                         const unsigned long long* volf, const unsigned long long* res, const unsigned long long* resd);
/* Tile shapes: threads per CTA of the face pass (64, 128, 256) and of the cell
 * passes (128, 256), CTAs per SM of the face pass (1..8); drops a captured graph. */
int bcg_batch_configure(long long plan, int tile_faces, int tile_cells, int ctas_per_sm);
/* Tile shapes of the chunks of host-array runs (bcg_batch_run_host) alone: a
 * chunk holds a few grids and runs beside the copies and the other chunks, so
 * its best shapes can differ from the whole batch's; once set, later
 * bcg_batch_configure calls no longer change them. */
int bcg_batch_configure_host(long long plan, int tile_faces, int tile_cells, int ctas_per_sm);
/* Queue one evaluation on the library stream; use_graph = 1 captures the
 * launches into a CUDA graph on first use and replays it afterwards. */
int bcg_batch_run(long long plan, int use_graph);
/* Queue one pass of an evaluation alone, outside any graph (0 primitives,
 * 1 Ducros gradients, 2 interpolation rows, 3 viscous point values, 4 faces,
 * 5 balance; run in that order they equal bcg_batch_run): for timing each
 * kernel of the evaluation with events on the library stream. */
int bcg_batch_run_pass(long long plan, int pass);
/* One evaluation with HOST arrays (tables of host addresses in the order of
 * bcg_batch_set_arrays; pinned memory copies fastest): the grids are split
 * into nchunk (1..16) contiguous chunks of about equal cell counts, and each
 * chunk's uploads (state, tangent, metrics), its graph replay and the
 * interior-only downloads of its residual and tangent overlap the other
 * chunks'.  The caller's ghost values of residu / residud stay untouched.
 * Returns when the outputs are in the host arrays.  The plan keeps device
 * mirrors of every grid's arrays after the first such call. */
int bcg_batch_run_host(long long plan, int nchunk, const unsigned long long* w, const unsigned long long* wd,
                       const unsigned long long* nx, const unsigned long long* ny, const unsigned long long* vol,
                       const unsigned long long* volf, const unsigned long long* res, const unsigned long long* resd);
int bcg_batch_device_bytes(long long plan, long long* bytes);
int bcg_batch_destroy(long long plan);

/* ---- allocation-free residual (no counterpart in the reference) --------------- */
/* For callers that cannot let the library allocate device memory during a call
 * (a framework allocator already owning the GPU's memory, a fixed memory
 * budget, loops that cannot absorb cudaMalloc's synchronisation).  Same
 * arguments and result as bcg_flux_num_dnc5_2d, but every array must be a
 * device pointer on the current device (-1 otherwise; -4 without a CUDA
 * device) and the working storage is a fixed 32 MiB static device
 * array (held by every GPU that loads the library until the process exits):
 * grids need 49*(im+6)*(jm+6) + 10*(im+1)*(jm+1) <= 4194304 doubles (256 x 256
 * and 400 x 150 fit); larger ones return -1.  All calls share that array:
 * calls that overlap on the GPU race, so serialise them.  The first call on a
 * device looks up the array's address for that device; make it before any
 * stream capture.  Queued on the library stream, returns without waiting. */
int bcg_flux_num_dnc5_2d_noalloc(double* residu, const double* w, const double* x0, const double* y0,
                                 const double* nx, const double* ny, const double* xc, const double* yc,
                                 const double* vol, const double* volf, int gh, double cp, double cv, double prandtl,
                                 double gam, double rgaz, double cs, double muref, double tref, double s_suth,
                                 double k2, double k4, int im, int jm);

/* ---- learned warm start (no reference counterpart) ----------------------------- */
/* Kernels of the conditioned MLP that gives the cylinder base-flow Newton
 * iteration (cylinder.py:841-1068) its initial state for a new (Re, Mach),
 * in place of the restart from a converged state on the same mesh
 * (cylinder.py:560-589).  BF16 operands (uint16 bit patterns), FP32
 * accumulation, row-major device arrays only; queued on the library stream.
 * GEMM  C[m x n] = A[m x k] B[n x k]^T (+ bias[n]), m and n multiples of 128,
 * k a multiple of 64, with the epilogue epi:
 *   0  out_bf = bf16(tanh(C))
 *   1  out_bf = bf16(C * (1 - yprev^2))              (backward through tanh)
 *   2  out_f32[m x nout] = C[:, :nout] (if given); with target [m x nout]:
 *      out_bf = bf16(gscale (C - target)) on the first nout columns of the
 *      first m_valid rows, 0 elsewhere, and loss_part[one per CTA] = the sum
 *      of squares of (C - target) there. */
int bcg_mlp_gemm_nn(int epi, const void* a, const void* b, const float* bias, const void* yprev, const float* target,
                    void* out_bf, float* out_f32, float* loss_part, int m, int n, int k, int nout, int m_valid,
                    float gscale);
/* part[z][n1 x n2] = sum over the rows of chunk z (m / nsplit rows, a multiple
 * of 64) of dz[row][n1] x[row][n2]; n1, n2 multiples of 128. */
int bcg_mlp_gemm_tn(const void* dz, const void* x, float* part, int m, int n1, int n2, int nsplit);
/* part[z][col] = sum of dz[row][col] over the rows of chunk z (ceil(m / nsplit) rows). */
int bcg_mlp_colsum(const void* dz, int m, int n, int nsplit, float* part);
/* gradient = fixed-order sum of the partials (weights n1 x n2, then bias n1),
 * written to grad_out if given; lr != 0: one Adam step on the FP32 master
 * weights and moments (lr carrying the bias corrections), refreshing the BF16
 * weights wbf [n1 x n2] and their transpose wtbf [n2 x n1]. */
int bcg_mlp_adam(const float* wpart, int nsplit, const float* bpart, int bsplit, int n1, int n2, float* w, float* mw,
                 float* vw, float* b, float* mb, float* vb, void* wbf, void* wtbf, float lr, float beta1, float beta2,
                 float eps, float* grad_out);
/* wbf = bf16(w) and wtbf its transpose. */
int bcg_mlp_cast_weights(const float* w, int n1, int n2, void* wbf, void* wtbf);
/* 128 BF16 input features per row of x [m x 128] from the cell's azimuth and
 * normalised log radius and the normalised (Re, Mach) of its parameter set.
 * seed >= 0: row r samples (set, cell) by a hash of (seed, r) and gathers its
 * targets [nset x ncell x nout] into t; seed < 0: row r is cell r of `set`.
 * Rows >= m_valid are zero. */
int bcg_mlp_features(const float* theta, const float* rho, int ncell, const float* params, int nset,
                     const float* targets, int nout, long long seed, int set, int m, int m_valid, void* x, float* t);
/* *out = sum of x[0..n) (one CTA, fixed order). */
int bcg_mlp_sum(const float* x, int n, float* out);

/* ---- calibration (no reference counterpart) ------------------------------------ */
/* FP64 FMA throughput of the current GPU in TFLOP/s (FMA = 2 flops): the
 * denominator of the FP64 roofline that bounds the residual kernels. */
int bcg_fp64_peak_tflops(double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* BROADCAST_GB300_H */
