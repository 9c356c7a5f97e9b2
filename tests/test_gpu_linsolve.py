"""The GPU band LU (bcg_csr_band_lu_solve) against scipy's sparse LU: random
banded systems that need pivoting, odd block sizes, the boundary-layer Newton
matrix, and a singular matrix."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _banded(n, kl, ku, seed, swapped=False):
    """Random diagonally dominant band matrix (sparse bands); swapped: its rows
    2k and 2k+1 interchanged, so that the diagonal holds small entries and
    partial pivoting must swap them back (bandwidths grow by one, the
    conditioning stays that of the dominant matrix)."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    rows, cols = [], []
    for d in range(-kl, ku + 1):
        i = np.arange(max(0, -d), min(n, n - d))
        keep = rng.random(i.size) < 0.6 if d != 0 else np.ones(i.size, bool)
        rows.append(i[keep])
        cols.append(i[keep] + d)
    r, c = np.concatenate(rows), np.concatenate(cols)
    v = rng.standard_normal(r.size)
    off = np.bincount(r[r != c], weights=np.abs(v[r != c]), minlength=n)  # strict row dominance
    diag = r == c
    v[diag] = np.sign(v[diag]) * (off[r[diag]] + 1.0)
    if swapped:
        r = np.where(r % 2 == 0, np.minimum(r + 1, n - 1) if n % 2 == 0 else np.where(r + 1 < n, r + 1, r),
                     r - 1)
    return sp.csr_matrix((v, (r, c)), shape=(n, n))


@pytest.mark.parametrize("n,kl,ku,nb,swapped", [(2000, 30, 25, 128, False), (1532, 17, 40, 7, True),
                                                (300, 60, 3, 64, True), (5, 2, 1, 128, False)])
def test_band_lu_matches_scipy(n, kl, ku, nb, swapped):
    from scipy.sparse.linalg import spsolve
    from broadcast_gb300.linsolve import band_lu_solve
    A = _banded(n, kl, ku, seed=n, swapped=swapped)
    b = np.random.default_rng(1).standard_normal(n)
    x = band_lu_solve(A, b, nb=nb)
    ref = spsolve(A.tocsc(), b)
    assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)
    assert np.abs(x - ref).max() <= 1e-8 * np.abs(ref).max()


def test_band_lu_newton_matrix():
    """The relaxed boundary-layer Jacobian of the Newton iteration (CSR from the
    GPU assembly) solved on the GPU and by SuperLU on the host."""
    from broadcast_gb300.linsolve import band_lu_solve
    from broadcast_gb300.newton import BLNewton, superlu_solve
    from tests import helpers as H
    c = H.bl_case(24, 16)
    nt = BLNewton(c, cfl=10.0)
    w = c["w"].copy(order="F")
    nt.fill(w)
    res, norm, _ = nt.residual(w)
    gh = c["grid"]["gh"]
    J = nt.jacobian(w, 0.1 * c["grid"]["vol"][gh:-gh, gh:-gh])
    rhs = np.ravel(res[gh:-gh, gh:-gh, :])
    x = band_lu_solve(J, rhs)
    ref = superlu_solve(J, rhs)
    assert np.abs(x - ref).max() <= 1e-10 * np.abs(ref).max()


def test_band_lu_singular():
    import scipy.sparse as sp
    from broadcast_gb300.linsolve import band_lu_solve
    A = sp.csr_matrix(np.array([[1.0, 2.0, 0.0], [2.0, 4.0, 0.0], [0.0, 0.0, 1.0]]))
    with pytest.raises(RuntimeError):
        band_lu_solve(A, np.ones(3))
