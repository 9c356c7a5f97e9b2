"""Linear solves of the Newton iteration on the GPU.

Two solvers: `band_lu_solve` (FP64 band LU, direct) and `KrylovSolver` (FP64
GMRES preconditioned by an FP32 band LU kept on the device and reused while it
keeps GMRES short; the large O-meshes, where FP64 factorisations cost minutes).

The reference factorises the Newton matrix with PETSc/MUMPS on the host
(BROADCAST_npz.py:1146-1158, misc/PETSc_func.py:137-152).  `band_lu_solve`
factorises it on the GPU instead: the boundary-layer Jacobian rows are ordered
(i, j, e) with i slowest, so the matrix is banded with bandwidth ~15 jm, and a
blocked band LU with partial pivoting (bcg_csr_band_lu_solve) is a direct
solve of the same accuracy class as MUMPS's LU.  It needs 8 n (3 kl + ku + 2 nb
+ 1) bytes of device memory (17 GB for the 400 x 150 boundary layer).
The trailing updates are DGEMMs of kl x (kl + ku) x nb, which cuBLAS runs at
~1.05 TFLOP/s on GB300 (its FP64 GEMM ceiling is ~1.1), so a factorisation
costs about 2 n kl (kl + ku) / 1.05e12 s plus the panels.
"""
import numpy as np

from . import _lib


def band_lu_solve(A, b, nb=256, perm=None):
    """x = A^-1 b for a scipy sparse matrix A (converted to CSR) and vector b.

    perm: optional bandwidth-reducing order (row/column k of A is factorised
    as row/column perm[k]).  Raises RuntimeError for a singular matrix (as
    scipy's splu does)."""
    A = A.tocsr()
    n = A.shape[0]
    indptr = np.ascontiguousarray(A.indptr, dtype=np.int32)
    indices = np.ascontiguousarray(A.indices, dtype=np.int32)
    data = np.ascontiguousarray(A.data, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n)
    info = np.zeros(1, np.int32)
    try:
        q = None if perm is None else np.ascontiguousarray(perm, dtype=np.int32)
        _lib.call("bcg_csr_band_lu_solve", n, indptr, indices, data, int(A.nnz), q, b, x, int(nb), info)
    except _lib.BroadcastError as e:
        if "singular" in str(e):
            raise RuntimeError("singular matrix (zero pivot at row %d)" % int(info[0])) from e
        raise
    return x


def folded_ring_order(im, jm, nvar=5):
    """Bandwidth-reducing order for the periodic O-mesh Jacobian (rows (i, j, e)
    with i slowest, i periodic): the azimuthal index folded (1, im, 2, im-1,
    ...) so that the periodic neighbours are close, and the radial index j
    slowest; returns perm with perm[row] = new position."""
    i = np.arange(im)
    fold = np.where(i < (im + 1) // 2, 2 * i, 2 * (im - 1 - i) + 1)  # 0, 2, 4, ..., 5, 3, 1
    ii, jj, ee = np.meshgrid(i, np.arange(jm), np.arange(nvar), indexing="ij")
    return (ee + nvar * fold[ii] + nvar * im * jj).ravel().astype(np.int32)


class KrylovSolver:
    """Newton-system solves on the GPU by FP64 GMRES (bcg_gmres_solve), right-
    preconditioned by an FP32 band LU of a recent Newton matrix
    (bcg_band32_factor: the row-equilibrated matrix in FP32, factorised in the
    bandwidth-reducing order perm).  The factor is reused for later systems
    (the next Newton steps, neighbouring base flows) and rebuilt from the
    current matrix when GMRES with it does not reach `rtol` within the
    iterations one factorisation costs (at least `refactor_after`).

    solve(indptr, indices, data, b) takes device tensors (torch, CSR int32 /
    float64) and returns x as a device tensor."""

    device_csr = True

    def __init__(self, perm=None, nb=1024, restart=60, maxit=400, rtol=1e-10, refactor_after=40):
        _lib.load()
        self.perm = None if perm is None else np.ascontiguousarray(perm, dtype=np.int32)
        self.nb, self.restart, self.maxit, self.rtol = int(nb), int(restart), int(maxit), float(rtol)
        self.refactor_after = int(refactor_after)
        self.handle = None
        self.n = None
        self.log = []
        self._perm_dev = None

    def close(self):
        if self.handle is not None:
            try:
                _lib.call("bcg_band32_destroy", self.handle)
            finally:
                self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def factor(self, indptr, indices, data):
        import torch
        self.close()
        n = int(indptr.numel()) - 1
        if self.perm is not None and self._perm_dev is None:
            self._perm_dev = torch.from_numpy(self.perm).to(indptr.device)
        h, info = np.zeros(1, np.int64), np.zeros(1, np.int32)
        try:
            _lib.call("bcg_band32_factor", n, indptr, indices, data, self._perm_dev, self.nb, h, info)
        except _lib.BroadcastError as e:
            if "singular" in str(e):
                raise RuntimeError("singular FP32 factor (zero pivot at row %d)" % int(info[0])) from e
            raise
        self.handle, self.n = int(h[0]), n

    def gmres(self, indptr, indices, data, b, x, maxit=None):
        it, rr = np.zeros(1, np.int32), np.zeros(1)
        _lib.call("bcg_gmres_solve", self.handle, self.n, indptr, indices, data, b, x, self.restart,
                  int(maxit or self.maxit), self.rtol, it, rr)
        return int(it[0]), float(rr[0])

    def solve(self, indptr, indices, data, b):
        """x with ||b - A x|| <= rtol ||b||.  With a kept factor, GMRES may run
        as many iterations as one factorisation costs (measured), at least
        refactor_after; past that, or if it stalls, the factor is rebuilt from
        this matrix and GMRES restarts."""
        import time
        import torch
        x = torch.empty_like(b)
        n = int(indptr.numel()) - 1
        t0 = time.perf_counter()
        refactored = False
        if self.handle is None or self.n != n:
            self.factor(indptr, indices, data)
            self._t_factor = time.perf_counter() - t0
            refactored = True
        t1 = time.perf_counter()
        budget = self.maxit
        if not refactored and getattr(self, "_t_iter", None):
            budget = int(np.clip(self._t_factor / self._t_iter, self.refactor_after, self.maxit))
        it, rr = self.gmres(indptr, indices, data, b, x, maxit=budget)
        if it:
            self._t_iter = (time.perf_counter() - t1) / it
        if not refactored and rr > self.rtol:
            tf = time.perf_counter()
            self.factor(indptr, indices, data)
            self._t_factor = time.perf_counter() - tf
            refactored = True
            t1 = time.perf_counter()
            it2, rr = self.gmres(indptr, indices, data, b, x)
            it += it2
        t2 = time.perf_counter()
        self.log.append(dict(iterations=it, relres=rr, refactored=refactored, seconds_factor=t1 - t0,
                             seconds_gmres=t2 - t1))
        if not (rr <= self.rtol * 10) or not torch.isfinite(x).all():
            raise RuntimeError("GMRES did not converge: relative residual %.2e after %d iterations" % (rr, it))
        return x
