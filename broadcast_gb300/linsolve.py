"""Linear solves of the Newton iteration on the GPU.

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
