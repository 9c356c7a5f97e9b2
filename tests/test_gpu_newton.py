"""SER Newton to a steady boundary layer (broadcast_gb300.newton): the first
update against the reference loop run through the oracle (relaxed Jacobian
from the per-seed loop, BROADCAST_npz.py:1068-1158, solved with the same
SuperLU), then convergence of the residual norm over the iterations."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _case():
    # a plate of 2e4 (Reynolds-number units) on 32 x 32 cells: the boundary
    # layer is resolved, so the Blasius start lies in Newton's basin
    return H.bl_case(32, 32, length=2.0e4)


def test_first_update_matches_reference_loop():
    sp = pytest.importorskip("scipy.sparse")
    from broadcast_gb300.newton import BLNewton, superlu_solve
    c = _case()
    nt = BLNewton(c, cfl=1.0, mach=0.5)  # a small CFL: the relaxation term is exercised
    w = c["w"].copy(order="F")
    w_before = w.copy(order="F")
    norm, dw = nt.step(w, first=True)
    # the reference loop through the oracle on the same filled state
    g, ph = c["grid"], c["phys"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    wf = w_before.copy(order="F")
    H.oracle_bcs(c, wf)
    res = O.residual(g, ph, wf)
    n2, ninf = O.norml2inf(res, im, jm, gh)
    n2, ninf = np.asarray(n2), np.asarray(ninf)
    r = np.max(np.concatenate([n2[:3] / np.maximum(n2[:3], 1e-15), ninf[:3] / np.maximum(ninf[:3], 1e-15)]))
    coef = np.asfortranarray(r * (1.0 / nt.dt) * g["vol"][gh:-gh, gh:-gh])
    nb = im * jm * 49 * 25
    jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
    for m in range(5):
        for l in range(7):
            for k in range(7):
                wd = O.testvector(m, l, k, gh, im, jm)
                H.oracle_bcs(c, wf.copy(order="F"), wd)
                _, resd = O.jvp(g, ph, wf, wd)
                O.computejacobian(O.JAC_RELAXED, jac, ia, ja, resd, m, l, k, gh, im, jm, coef)
    keep = np.abs(jac) > 2e-16
    J = sp.csr_matrix((jac[keep], (ia[keep], ja[keep])), shape=(5 * im * jm, 5 * im * jm))
    ref = np.reshape(superlu_solve(J, np.ravel(res[gh:-gh, gh:-gh, :])), (im, jm, 5))
    assert np.abs(dw - ref).max() <= 1e-9 * np.abs(ref).max()
    assert np.allclose(norm, n2, rtol=1e-11, atol=0)


def test_newton_converges():
    from broadcast_gb300.newton import BLNewton
    c = _case()
    nt = BLNewton(c, mach=0.5)  # cfl = 1e10 as the reference card: Newton's method
    w = c["w"].copy(order="F")
    nt.solve(w, ite=12, tol=1e-10)
    norms = np.array([h["norm"] for h in nt.history]).max(axis=1)
    assert norms[-1] <= 1e-10, norms          # converged (absolute L2 norm, the bar of the reference's C5)
    assert len(nt.history) <= 8, norms        # quadratic convergence: 6 iterations on the CPU oracle


def test_cylinder_first_update_matches_reference_loop():
    """cylinder.py:841-1068: the first update (cfl 0.9 as the cylinder card,
    so the relaxation is exercised) against the reference loop through the
    oracle (relaxed, periodic column wrap, SuperLU); the GPU solve is the band
    LU in the folded azimuthal order."""
    sp = pytest.importorskip("scipy.sparse")
    from broadcast_gb300.newton import CylNewton, superlu_solve
    c = H.cyl_case(28, 21)
    nt = CylNewton(c, cfl=0.9)
    w = c["w"].copy(order="F")
    w_before = w.copy(order="F")
    norm, dw = nt.step(w, first=True)
    g, ph = c["grid"], c["phys"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    wf = w_before.copy(order="F")
    H.oracle_bcs(c, wf)
    res = O.residual(g, ph, wf)
    n2, ninf = O.norml2inf(res, im, jm, gh)
    coef = np.asfortranarray(1.0 / nt.dt * g["vol"][gh:-gh, gh:-gh])  # r = 1 at the first iterate
    nb = im * jm * 49 * 25
    jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
    for m in range(5):
        for l in range(7):
            for k in range(7):
                wd = O.testvector(m, l, k, gh, im, jm)
                H.oracle_bcs(c, wf.copy(order="F"), wd)
                _, resd = O.jvp(g, ph, wf, wd)
                O.computejacobian(O.JAC_RELAXED_WITHJN, jac, ia, ja, resd, m, l, k, gh, im, jm, coef)
    keep = np.abs(jac) > 2e-16
    J = sp.csr_matrix((jac[keep], (ia[keep], ja[keep])), shape=(5 * im * jm, 5 * im * jm))
    ref = np.reshape(superlu_solve(J, np.ravel(res[gh:-gh, gh:-gh, :])), (im, jm, 5))
    assert np.abs(dw - ref).max() <= 1e-9 * np.abs(ref).max()
    assert np.allclose(norm, np.asarray(n2), rtol=1e-11, atol=0)


def test_cylinder_newton_converges():
    """Newton's iteration (cfl 1e10) from the uniform flow converges
    quadratically: 6 iterations to 1.4e-11 in the oracle prototype."""
    from broadcast_gb300.newton import CylNewton
    c = H.cyl_case(28, 21)
    nt = CylNewton(c)
    w = c["w"].copy(order="F")
    nt.solve(w, ite=12, tol=1e-10)
    norms = np.array([h["norm"] for h in nt.history]).max(axis=1)
    assert norms[-1] <= 1e-10, norms
    assert len(nt.history) <= 8, norms


def test_folded_order_band_lu_matches_superlu():
    """The periodic Jacobian solved by the band LU with and without the folded
    order (bandwidth 15 im + 35 instead of ~5 jm im) and by SuperLU."""
    from broadcast_gb300.linsolve import band_lu_solve, folded_ring_order
    from broadcast_gb300.newton import CylNewton, superlu_solve
    c = H.cyl_case(28, 21)
    nt = CylNewton(c, cfl=5.0)
    w = c["w"].copy(order="F")
    nt.fill(w)
    res, _, _ = nt.residual(w)
    gh = 3
    J = nt.jacobian(w, 0.2 * c["grid"]["vol"][gh:-gh, gh:-gh])
    rhs = np.ravel(res[gh:-gh, gh:-gh, :])
    ref = superlu_solve(J, rhs)
    for perm in (folded_ring_order(28, 21), None):
        x = band_lu_solve(J, rhs, perm=perm)
        assert np.abs(x - ref).max() <= 1e-10 * np.abs(ref).max()
    bad = np.arange(J.shape[0], dtype=np.int32)
    bad[0] = 1  # not a permutation: refused before any launch
    with pytest.raises(Exception):
        band_lu_solve(J, rhs, perm=bad)
