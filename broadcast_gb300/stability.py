"""Global stability stage fed by the GPU-assembled matrices (the caller of the
hot path in biglobal.py:60-110 and biglobal_cyl.py:47-104).

For each spanwise wavenumber beta the operator J(beta) = J - beta^2 Dzz +
i beta Dz (biglobal.py:82) is formed on the GPU on the union pattern of the
three CSR matrices (bcg_csr_spanwise_beta), then the eigenvalues nearest a
target are found by shift-invert.  The reference does the shift-invert with
PETSc/MUMPS and SLEPc (misc/PETSc_func.py:1516-1539, eigPetsc3); those are
not installed here, so the solve runs through scipy's ARPACK with a SuperLU
factorisation, which fits grids up to a few hundred thousand unknowns.
"""
import numpy as np

from . import _lib


def spanwise_operators(J, Dz, Dzz, betas):
    """J(beta) for every beta, as scipy CSR complex matrices on the union pattern.

    J, Dz, Dzz: scipy CSR matrices (float64, sorted indices) of the same shape."""
    import scipy.sparse as sp
    nrow = J.shape[0]
    betas = np.ascontiguousarray(betas, dtype=np.float64)
    mats = [m.tocsr() for m in (J, Dz, Dzz)]
    for m in mats:
        m.sort_indices()
    cap = sum(m.nnz for m in mats)
    indptr, indices = np.zeros(nrow + 1, np.int32), np.zeros(cap, np.int32)
    vals = np.zeros(2 * len(betas) * cap)
    nnz = np.zeros(1, np.int64)
    args = []
    for m in mats:
        args += [np.ascontiguousarray(m.indptr, dtype=np.int32), np.ascontiguousarray(m.indices, dtype=np.int32),
                 np.ascontiguousarray(m.data, dtype=np.float64)]
    _lib.call("bcg_csr_spanwise_beta", nrow, *args, len(betas), betas, indptr, indices, vals, cap, nnz)
    n = int(nnz[0])
    cv = vals[:2 * len(betas) * n].reshape(len(betas), n, 2)
    return [sp.csr_matrix((cv[k, :, 0] + 1j * cv[k, :, 1], indices[:n].copy(), indptr.copy()), shape=J.shape)
            for k in range(len(betas))]


def leading_eigenvalues(A, target, nev=10, tol=1e-12):
    """Eigenvalues of A nearest `target` (shift-invert), sorted by distance to it."""
    from scipy.sparse.linalg import eigs
    vals = eigs(A.tocsc(), k=nev, sigma=target, which="LM", tol=tol, return_eigenvectors=False)
    return vals[np.argsort(np.abs(vals - target))]


def spectrum(J, Dz, Dzz, betas, target, nev=10):
    """Leading eigenvalues per beta: array (len(betas), nev)."""
    return np.stack([leading_eigenvalues(A, target, nev) for A in spanwise_operators(J, Dz, Dzz, betas)])
