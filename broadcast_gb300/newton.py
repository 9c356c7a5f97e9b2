"""Pseudo-transient Newton (SER) iteration to a steady base flow: the
'fixed_point' mode of the boundary-layer driver (BROADCAST_npz.py:985-1196,
BLNewton) and of the cylinder driver (cylinder.py:841-1068, CylNewton), the
immediate callers of the residual and Jacobian hot path.

Per iteration, as the reference:
  1. boundary fills (inlet Ilo, no-reflexion Jhi, extrapolation Ihi, wall Jlo);
  2. residual R(w) and its L2 / L10 norms (srcfv/norm.F90);
  3. relaxation 1/cfl = r / dt with r = max of the first three normalised norms
     (:1079-1087) and coefdiag = (1/cfl) vol;
  4. the relaxed Jacobian coefdiag - dR/dw for all 245 colour seeds as CSR
     (computejacobianfromjv_relaxed + remove_zero_jac, :1088-1137);
  5. solve J dw = R (:1146-1158: PETSc LU with MUMPS there) and w += dw,
     stepping back and halving cfl when dw is not finite (:1167-1172).
Steps 1, 2 and 4 run on the GPU through the library; step 5 calls `solver`,
by default the GPU band LU (broadcast_gb300.linsolve.band_lu_solve: the
Jacobian is banded with bandwidth ~15 jm in its (i, j, e) row order); a
linsolve.KrylovSolver (FP64 GMRES preconditioned by a reused FP32 band LU,
the matrix assembled straight into device memory) for large grids;
`superlu_solve` (scipy, host) or a PETSc/MUMPS solve can be passed instead.
"""
import time

import numpy as np

from . import _lib
from .linsolve import band_lu_solve, folded_ring_order

PHYS = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")


def superlu_solve(A, b):
    from scipy.sparse.linalg import splu
    return splu(A.tocsc(), permc_spec="COLAMD").solve(b)


class BLNewton:
    """SER Newton on a boundary-layer case (broadcast_gb300.cases.bl_case layout);
    cfl = 1e10 is the boundary-layer card's setting (card_bl2d_fv_npz.py:56):
    the relaxation vanishes and the iteration is Newton's."""

    # the boundary-layer driver forms dt once, before its Newton loop
    # (BROADCAST_npz.py:1009): halving the CFL number after a failed update
    # leaves dt as it was; the cylinder driver forms dt from the CFL number at
    # every iteration (cylinder.py:842), so there dt halves with it
    dt_follows_cfl = False

    def __init__(self, case, cfl=1.0e10, mach=None, solver=band_lu_solve):
        from ._f2py import interf4
        _lib.load()
        self.c = case
        g, ph = case["grid"], case["phys"]
        self.im, self.jm, self.gh = int(g["im"]), int(g["jm"]), int(g["gh"])
        self.phys = [float(ph[k]) for k in PHYS]
        self.mach = float(mach if mach is not None else ph.get("mach", 0.5))
        self.cfl = float(cfl)
        if solver == "krylov":  # FP64 GMRES with a reused FP32 band LU preconditioner
            from .linsolve import KrylovSolver
            solver = KrylovSolver()
        self.solver = solver
        it = case["interf"]
        self.interf = [interf4(it[k]) for k in ("Ilo", "Jhi", "Ihi", "Jlo")]
        yc = g["yc"]
        gh = self.gh
        self.dt = self.cfl * (yc[gh, gh + 1] - yc[gh, gh]) / (1.0 / self.mach + 1.0)
        self.history = []

    def fill(self, w):
        from .srcfv import f_bnd
        c, g = self.c, self.c["grid"]
        it, gam = c["interf"], self.c["phys"]["gam"]
        f_bnd.bc_supandsubinlet_2d(w, "Ilo", it["Ilo"], c["field"], g["nx"], g["ny"], gam, self.im, self.jm)
        f_bnd.bc_no_reflexion_2d(w, c["wbd"], "Jhi", it["Jhi"], g["nx"], g["ny"], gam, self.gh, self.im, self.jm)
        f_bnd.bc_extrapolate_o2_2d(w, "Ihi", it["Ihi"], self.im, self.jm, self.gh)
        f_bnd.bc_wall_viscous_adia_2d(w, "Jlo", gam, it["Jlo"], self.gh, self.im, self.jm)

    def residual(self, w):
        from .srcfv import f_norm, f_sch
        g = self.c["grid"]
        res = np.zeros_like(w)
        f_sch.flux_num_dnc5_2d(res, w, g["x0"], g["y0"], g["nx"], g["ny"], g["xc"], g["yc"], g["vol"], g["volf"],
                               self.gh, *self.phys, self.im, self.jm)
        norm, ninf = f_norm.compute_norml2inf(res, self.im, self.jm, self.gh)
        return res, np.asarray(norm), np.asarray(ninf)

    def _jac_args(self, w, coefdiag):
        g, c = self.c["grid"], self.c
        return ("bcg_jacobian_dnc5_bl_csr", (w, g["nx"], g["ny"], g["vol"], g["volf"], self.gh, *self.phys, self.im,
                                             self.jm, *self.interf, c["field"], c["field"].shape[0], c["wbd"],
                                             c["wbd"].shape[0], np.asfortranarray(coefdiag), 2e-16, 0))

    def jacobian(self, w, coefdiag):
        import scipy.sparse as sp
        nrow = 5 * self.im * self.jm
        cap = nrow * 245
        indptr, indices, data = np.zeros(nrow + 1, np.int32), np.zeros(cap, np.int32), np.zeros(cap)
        nnz = np.zeros(1, np.int64)
        name, args = self._jac_args(w, coefdiag)
        _lib.call(name, *args, indptr, indices, data, cap, nnz)
        n = int(nnz[0])
        return sp.csr_matrix((data[:n].copy(), indices[:n].copy(), indptr), shape=(nrow, nrow))

    def jacobian_device(self, w, coefdiag):
        """The same CSR matrix in device tensors (indptr, indices, data)."""
        import torch
        nrow = 5 * self.im * self.jm
        cap = nrow * 245
        dev = torch.device("cuda", torch.cuda.current_device())
        if getattr(self, "_jbuf", None) is None or self._jbuf[1].numel() != cap:
            self._jbuf = (torch.empty(nrow + 1, dtype=torch.int32, device=dev),
                          torch.empty(cap, dtype=torch.int32, device=dev),
                          torch.empty(cap, dtype=torch.float64, device=dev))
        indptr, indices, data = self._jbuf
        nnz = np.zeros(1, np.int64)
        _lib.call("bcg_set_stream", torch.cuda.current_stream(dev).cuda_stream)
        name, args = self._jac_args(w, coefdiag)
        _lib.call(name, *args, indptr, indices, data, cap, nnz)
        n = int(nnz[0])
        return indptr, indices[:n], data[:n]

    def step(self, w, first=False, tol=None):
        """One SER Newton iteration on w (Fortran-ordered, updated in place).
        With tol given, a state whose max L2 residual norm is already <= tol
        is left as it is (no Jacobian, no solve) and dw is None."""
        t0 = time.perf_counter()
        self.fill(w)
        res, norm, ninf = self.residual(w)
        t1 = time.perf_counter()
        if tol is not None and norm.max() <= tol:
            self.history.append(dict(norm=norm.tolist(), cflm1=0.0, nnz=0, seconds=t1 - t0, seconds_residual=t1 - t0,
                                     seconds_jacobian=0.0, seconds_solve=0.0))
            return norm, None
        if first:
            self.norm0m1 = 1.0 / np.maximum(norm, 1e-15)
            self.ninf0m1 = 1.0 / np.maximum(ninf, 1e-15)
        r = np.max(np.concatenate([norm[:3] * self.norm0m1[:3], ninf[:3] * self.ninf0m1[:3]]))
        dtm1 = 1.0 / self.dt
        cflm1 = r * dtm1  # BROADCAST_npz.py:1010,1063; cylinder.py:843,890
        gh = self.gh
        coefdiag = cflm1 * self.c["grid"]["vol"][gh:-gh, gh:-gh]
        rhs = np.ravel(res[gh:-gh, gh:-gh, :])
        if getattr(self.solver, "device_csr", False):  # GPU matrix and solve (KrylovSolver)
            import torch
            J = self.jacobian_device(w, coefdiag)
            t2 = time.perf_counter()
            try:
                x = self.solver.solve(*J, torch.from_numpy(rhs).to(J[0].device))
                dw = np.reshape(x.cpu().numpy(), (self.im, self.jm, 5))
            except RuntimeError:  # singular factor or no convergence: treated like a non-finite update
                dw = np.full((self.im, self.jm, 5), np.nan)
            nnz = int(J[2].numel())
        else:
            J = self.jacobian(w, coefdiag)
            t2 = time.perf_counter()
            try:
                dw = np.reshape(self.solver(J, rhs), (self.im, self.jm, 5))
            except RuntimeError:  # singular factorisation: treated like a non-finite update
                dw = np.full((self.im, self.jm, 5), np.nan)
            nnz = int(J.nnz)
        if np.all(np.isfinite(dw)):
            w[gh:-gh, gh:-gh, :] += dw
            self.dw_old = dw
        else:
            # step back and halve the CFL number (BROADCAST_npz.py:1170-1175,
            # cylinder.py:1026-1031)
            if hasattr(self, "dw_old"):
                w[gh:-gh, gh:-gh, :] -= self.dw_old
            self.cfl /= 2.0
            if self.dt_follows_cfl:
                self.dt /= 2.0
        t3 = time.perf_counter()
        self.history.append(dict(norm=norm.tolist(), cflm1=float(cflm1), nnz=nnz, seconds=t3 - t0,
                                 seconds_residual=t1 - t0, seconds_jacobian=t2 - t1, seconds_solve=t3 - t2))
        return norm, dw

    def solve(self, w, ite=50, tol=1e-10):
        """Iterate until max L2 residual norm <= tol (absolute) or ite steps."""
        for it in range(1, ite + 1):
            norm, dw = self.step(w, first=(it == 1), tol=tol)
            if dw is None:
                break
        self.fill(w)
        return w


class CylNewton(BLNewton):
    """SER Newton on the cylinder O-mesh (broadcast_gb300.cases.cyl_case layout),
    cylinder.py:841-1068: boundary fills no-reflexion (Jhi), wall (Jlo) and
    the two periodic joins in handleBC.applyBC's order; time step from the
    radial spacing of the first cell, dt = cfl |xc(1,1) - xc(1,2)| / (1/M + 1)
    (:842); relaxed Jacobian with the periodic column wrap
    (computejacobianfromjv_relaxed_withjn[andcheck], :900-980) assembled on the
    GPU; the linear solve by the GPU band LU in the folded azimuthal order,
    which makes the periodic Jacobian banded (kl ~ 15 im + 35).  The cylinder
    card runs cfl 0.9 (card_cyl2d.py:57); cfl 1e10 gives Newton's iteration."""

    dt_follows_cfl = True

    def __init__(self, case, cfl=1.0e10, mach=None, solver=None):
        g = case["grid"]
        self.perm = folded_ring_order(int(g["im"]), int(g["jm"]))
        if solver == "krylov":  # FP64 GMRES, FP32 band LU preconditioner in the folded order
            from .linsolve import KrylovSolver
            solver = KrylovSolver(perm=self.perm)
        super().__init__(case, cfl=cfl, mach=mach, solver=solver or self._banded)
        gh = self.gh
        self.dt = self.cfl * abs(g["xc"][gh, gh] - g["xc"][gh, gh + 1]) / (1.0 / self.mach + 1.0)

    def _banded(self, J, b):
        return band_lu_solve(J, b, perm=self.perm)

    def fill(self, w):
        from .srcfv import f_bnd
        c, g = self.c, self.c["grid"]
        it, gam, gh, im, jm = c["interf"], self.c["phys"]["gam"], self.gh, self.im, self.jm
        f_bnd.bc_no_reflexion_2d(w, c["wbd"], "Jhi", it["Jhi"], g["nx"], g["ny"], gam, gh, im, jm)
        f_bnd.bc_wall_viscous_adia_2d(w, "Jlo", gam, it["Jlo"], gh, im, jm)
        for _ in range(2):  # the joins of interf3 and interf4 each apply both copies
            f_bnd.jn_match_2d(w, it["prr1"], gh, gh, gh, gh, im, jm, w, it["prd2"], gh, gh, gh, gh, im, jm, it["tr"])
            f_bnd.jn_match_2d(w, it["prr2"], gh, gh, gh, gh, im, jm, w, it["prd1"], gh, gh, gh, gh, im, jm, it["tr"])

    def _jac_args(self, w, coefdiag):
        from ._f2py import interf4
        g, c = self.c["grid"], self.c
        it = c["interf"]
        return ("bcg_jacobian_dnc5_cyl_csr", (w, g["nx"], g["ny"], g["vol"], g["volf"], self.gh, *self.phys, self.im,
                                              self.jm, interf4(it["Jhi"]), interf4(it["Jlo"]), c["wbd"],
                                              c["wbd"].shape[0], interf4(it["prr1"]), interf4(it["prd1"]),
                                              interf4(it["prr2"]), interf4(it["prd2"]),
                                              np.ascontiguousarray(np.asarray(it["tr"], dtype=np.int32).ravel()),
                                              np.asfortranarray(coefdiag), 2e-16, 0))
