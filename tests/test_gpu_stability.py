"""The stability stage fed by the GPU matrices against the same stage fed by
the reference's per-seed loop run through the oracle (BROADCAST_npz.py:
1068-1137, 1206-1210, 1221-1249): J/vol, Dz and Dzz of a small boundary
layer, J(beta) = J - beta^2 Dzz + i beta Dz (biglobal.py:82), ten eigenvalues
nearest a target by shift-invert.  Bar: 1e-8 relative.  PETSc /
SLEPc are absent, so both sides use scipy's ARPACK + SuperLU: this pins the
matrices handed to the eigen stage, not PETSc itself."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu
SPAN = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth")


def _reference_lists(c, kind):
    sp = pytest.importorskip("scipy.sparse")
    g = c["grid"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    nb = im * jm * 49 * 25
    jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
    for m in range(5):
        for l in range(7):
            for k in range(7):
                wd = O.testvector(m, l, k, gh, im, jm)
                H.oracle_bcs(c, c["w"].copy(order="F"), wd)
                if kind == "J":
                    _, out = O.jvp(g, c["phys"], c["w"], wd)
                    O.computejacobian(O.JAC_PLAIN, jac, ia, ja, out, m, l, k, gh, im, jm, None)
                else:
                    out = (O.dz if kind == "Dz" else O.dzz)(g, c["phys"], c["w"], wd)
                    O.computejacobian(O.JAC_DZ, jac, ia, ja, out, m, l, k, gh, im, jm, None)
    keep = np.abs(jac) > 2e-16
    jac, ia, ja = jac[keep], ia[keep], ja[keep]
    if kind == "J":  # Jacvol (BROADCAST_npz.py:1206-1210)
        jac = jac / g["vol"][(ia // (jm * 5)) + gh, ((ia % (jm * 5)) // 5) + gh]
    a = sp.csr_matrix((jac, (ia, ja)), shape=(5 * im * jm, 5 * im * jm))
    a.sort_indices()
    return a


def _gpu(c, kind):
    sp = pytest.importorskip("scipy.sparse")
    from broadcast_gb300 import _lib
    from broadcast_gb300._f2py import interf4
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    nrow = 5 * im * jm
    cap = nrow * 245
    indptr, indices, data = np.zeros(nrow + 1, np.int32), np.zeros(cap, np.int32), np.zeros(cap)
    nnz = np.zeros(1, np.int64)
    common = (interf4(it["Ilo"]), interf4(it["Jhi"]), interf4(it["Ihi"]), interf4(it["Jlo"]), c["field"],
              c["field"].shape[0], c["wbd"], c["wbd"].shape[0])
    if kind == "J":
        _lib.call("bcg_jacobian_dnc5_bl_csr", c["w"], g["nx"], g["ny"], g["vol"], g["volf"], gh,
                  *[float(ph[k]) for k in SPAN + ("k2", "k4")], im, jm, *common, None, 2e-16, 1, indptr, indices,
                  data, cap, nnz)
    else:
        _lib.call("bcg_jacobian_dz_bl_csr", c["w"], g["nx"], g["ny"], g["vol"], g["volf"], gh,
                  *[float(ph[k]) for k in SPAN], im, jm, *common, 1 if kind == "Dz" else 2, 2e-16, indptr, indices,
                  data, cap, nnz)
    n = int(nnz[0])
    return sp.csr_matrix((data[:n].copy(), indices[:n].copy(), indptr.copy()), shape=(nrow, nrow))


def test_leading_eigenvalues_match_reference_matrices():
    pytest.importorskip("scipy.sparse.linalg")
    from broadcast_gb300 import stability
    c = H.bl_case(16, 12)
    H.oracle_bcs(c, c["w"])
    gpu = [_gpu(c, k) for k in ("J", "Dz", "Dzz")]
    ref = [_reference_lists(c, k) for k in ("J", "Dz", "Dzz")]
    betas = [0.0, 0.5, 1.5]
    target = 0.05 + 0.05j
    got = stability.spectrum(*gpu, betas, target, nev=10)
    import scipy.sparse as sp
    for k, b in enumerate(betas):
        A = (ref[0] - b * b * ref[2] + 1j * b * ref[1]).tocsr()
        want = stability.leading_eigenvalues(A, target, nev=10)
        # match each eigenvalue to its nearest counterpart (clusters may swap order)
        dist = np.abs(got[k][:, None] - want[None, :]).min(axis=1)
        assert dist.max() <= 1e-8 * np.abs(want).max(), (b, got[k], want)
