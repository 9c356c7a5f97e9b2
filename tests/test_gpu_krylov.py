"""Newton-Krylov solves (linsolve.KrylovSolver: FP64 GMRES right-preconditioned
by an FP32 band LU of the row-equilibrated matrix, bcg_band32_factor /
bcg_gmres_solve): random band systems that need pivoting against scipy's LU,
the periodic O-mesh Newton matrix against the FP64 band LU in the folded
order, a factor reused for a neighbouring matrix, and Newton's iteration on a
boundary layer with the Krylov solve converging as with the direct one."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu


def _dev_csr(A):
    import torch
    A = A.tocsr()
    A.sort_indices()
    d = torch.device("cuda")
    return (torch.from_numpy(np.ascontiguousarray(A.indptr, dtype=np.int32)).to(d),
            torch.from_numpy(np.ascontiguousarray(A.indices, dtype=np.int32)).to(d),
            torch.from_numpy(np.ascontiguousarray(A.data, dtype=np.float64)).to(d))


@pytest.mark.parametrize("n,kl,ku,nb,swapped", [(2000, 30, 25, 128, False), (1532, 17, 40, 7, True),
                                                (300, 60, 3, 64, True)])
def test_gmres_band32_matches_scipy(n, kl, ku, nb, swapped):
    import torch
    from scipy.sparse.linalg import spsolve
    from broadcast_gb300.linsolve import KrylovSolver
    from tests.test_gpu_linsolve import _banded
    A = _banded(n, kl, ku, seed=n, swapped=swapped)
    b = np.random.default_rng(1).standard_normal(n)
    ks = KrylovSolver(nb=nb, rtol=1e-12)
    x = ks.solve(*_dev_csr(A), torch.from_numpy(b).cuda()).cpu().numpy()
    ref = spsolve(A.tocsc(), b)
    assert np.linalg.norm(A @ x - b) <= 1e-11 * np.linalg.norm(b)
    assert np.abs(x - ref).max() <= 1e-9 * np.abs(ref).max()
    assert ks.log[-1]["iterations"] <= 10   # an FP32 factor of the same matrix


def _cyl_matrix(im=28, jm=21, scale=1e-3, seed=4):
    """Newton matrix (cfl 1e10) of the periodic O-mesh at a perturbed uniform flow."""
    from broadcast_gb300.newton import CylNewton
    c = H.cyl_case(im, jm, noise=0.0)
    w = c["w"].copy(order="F")
    rng = np.random.default_rng(seed)
    w[3:-3, 3:-3] *= 1.0 + scale * rng.standard_normal((im, jm, 5))
    nt = CylNewton(c)
    nt.fill(w)
    res, _, _ = nt.residual(w)
    J = nt.jacobian(w, np.zeros((im, jm)))
    return nt, J, np.ravel(res[3:-3, 3:-3, :])


def test_cylinder_newton_matrix_and_factor_reuse():
    import torch
    from broadcast_gb300.linsolve import KrylovSolver, band_lu_solve
    nt, J, b = _cyl_matrix()
    ref = band_lu_solve(J, b, perm=nt.perm)
    ks = KrylovSolver(perm=nt.perm, rtol=1e-12)
    x = ks.solve(*_dev_csr(J), torch.from_numpy(b).cuda()).cpu().numpy()
    assert np.abs(x - ref).max() <= 1e-9 * np.abs(ref).max()
    assert ks.log[-1]["refactored"]
    # a neighbouring matrix (another perturbation) with the kept factor
    _, J2, b2 = _cyl_matrix(seed=5)
    ref2 = band_lu_solve(J2, b2, perm=nt.perm)
    x2 = ks.solve(*_dev_csr(J2), torch.from_numpy(b2).cuda()).cpu().numpy()
    assert not ks.log[-1]["refactored"]
    assert np.abs(x2 - ref2).max() <= 1e-9 * np.abs(ref2).max()
    dims = np.zeros(3, np.int32)
    from broadcast_gb300 import _lib
    _lib.call("bcg_band32_dims", ks.handle, dims)
    coo = J.tocoo()
    pr, pc = nt.perm[coo.row], nt.perm[coo.col]
    assert (dims[0], dims[1]) == (int((pr - pc).max()), int((pc - pr).max()))   # the folded order's band


def test_newton_with_krylov_converges_as_direct():
    from broadcast_gb300.newton import BLNewton
    c = H.bl_case(32, 32, length=2.0e4)
    norms = {}
    for solver in ("krylov", None):
        nt = BLNewton(c, mach=0.5) if solver is None else BLNewton(c, mach=0.5, solver=solver)
        w = c["w"].copy(order="F")
        nt.solve(w, ite=12, tol=1e-10)
        norms[solver] = np.array([h["norm"] for h in nt.history]).max(axis=1)
    assert norms["krylov"][-1] <= 1e-10 and norms[None][-1] <= 1e-10
    assert len(norms["krylov"]) == len(norms[None])
    assert np.allclose(norms["krylov"][:3], norms[None][:3], rtol=1e-6)


def test_bad_inputs_are_rejected():
    from broadcast_gb300 import _lib
    with pytest.raises(_lib.BroadcastError):
        _lib.call("bcg_band32_solve", 987654321, None, None)
    x = np.zeros(4)
    with pytest.raises(_lib.BroadcastError):  # host arrays
        _lib.call("bcg_gmres_solve", 1, 3, np.zeros(4, np.int32), np.zeros(1, np.int32), x, x, x, 10, 10, 1e-8,
                  np.zeros(1, np.int32), np.zeros(1))
