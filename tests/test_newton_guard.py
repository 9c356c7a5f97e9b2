"""The Newton iteration's failure guard, with the failure made on the host
(CPU only).

BROADCAST_npz.py:1170-1175 (and cylinder.py:1026-1031): when the update dw
has a NaN, the previous update is taken back from the state and the CFL number
is halved; the previous update is not replaced, so a second failure in a row
takes the same update back again.  The boundary-layer driver forms its time
step once, before the loop (BROADCAST_npz.py:1009), so the halved CFL number
leaves it unchanged; the cylinder driver forms it from the CFL number at every
iteration (cylinder.py:842), so there it halves.  BLNewton and CylNewton do the
same, and treat a singular factorisation or a solve that does not converge
like a non-finite update.
The residual, boundary fills and Jacobian are stubbed; the solver is a fake
that returns a finite update, then a NaN update, then raises.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from broadcast_gb300.newton import BLNewton, CylNewton


def _driver(solver, norms, cls=BLNewton):
    nw = object.__new__(cls)
    nw.gh, nw.im, nw.jm = 3, 6, 5
    nw.c = {"grid": {"vol": np.ones((12, 11), order="F")}}
    nw.cfl, nw.dt, nw.history = 10.0, 2.0, []
    nw.solver = solver
    calls = iter(norms)
    nw.fill = lambda w: None

    def residual(w):
        n = next(calls)
        return np.ones_like(w), np.full(5, n), np.full(5, n)

    nw.residual = residual
    nw.jacobian = lambda w, coefdiag: sp.identity(5 * nw.im * nw.jm, format="csr")
    return nw


@pytest.mark.parametrize("cls", [BLNewton, CylNewton])
def test_non_finite_update_steps_back_and_halves_the_cfl(cls):
    dw1 = np.full((6, 5, 5), 0.125)
    outcomes = [dw1.ravel(), np.full(150, np.nan), RuntimeError("singular pivot")]

    def solver(J, rhs):
        o = outcomes.pop(0)
        if isinstance(o, Exception):
            raise o
        return o

    nw = _driver(solver, [1.0, 0.5, 0.5, 1e-12], cls)
    halved = 0.5 if cls.dt_follows_cfl else 1.0
    w = np.asfortranarray(np.random.default_rng(0).uniform(1.0, 2.0, (12, 11, 5)))
    w0 = w.copy()
    inner = (slice(3, -3), slice(3, -3))

    _, dw = nw.step(w, first=True, tol=1e-10)                  # accepted
    assert np.array_equal(w[inner], w0[inner] + dw1) and np.array_equal(dw, dw1)
    assert (nw.cfl, nw.dt) == (10.0, 2.0)

    _, dw = nw.step(w, tol=1e-10)                              # NaN: back to w0, CFL halved
    assert not np.isfinite(dw).all()
    assert np.array_equal(w[inner], w0[inner] + dw1 - dw1)
    assert (nw.cfl, nw.dt) == (5.0, 2.0 * halved)

    _, dw = nw.step(w, tol=1e-10)                              # singular solve: the same update taken back again
    assert np.isnan(dw).all()
    assert np.array_equal(w[inner], w0[inner] + dw1 - dw1 - dw1)
    assert (nw.cfl, nw.dt) == (2.5, 2.0 * halved * halved)

    norm, dw = nw.step(w, tol=1e-10)                           # converged: nothing assembled or solved
    assert dw is None and norm.max() <= 1e-10 and outcomes == []
    assert np.array_equal(w[:3], w0[:3]) and np.array_equal(w[:, :3], w0[:, :3])   # ghosts untouched (fill stubbed)
    assert len(nw.history) == 4 and nw.history[-1]["nnz"] == 0


def test_first_step_failure_has_nothing_to_take_back():
    nw = _driver(lambda J, rhs: np.full(150, np.inf), [1.0])
    w = np.asfortranarray(np.ones((12, 11, 5)))
    nw.step(w, first=True, tol=1e-10)
    assert np.array_equal(w, np.ones((12, 11, 5))) and nw.cfl == 5.0
    with pytest.raises(AttributeError):
        nw.dw_old
