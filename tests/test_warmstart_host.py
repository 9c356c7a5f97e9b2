"""CPU checks of the learned warm start's host logic with a stand-in for the
GPU Newton iteration: the continuation order of the base-flow generation,
its retry by grid sequencing from the uniform flow, the plain / learned
comparison with its fallbacks, and the grid sequence's levels and state
interpolation between O-meshes."""
import numpy as np
import pytest

from broadcast_gb300 import warmstart as WS

IM, JM = 12, 10


def _truth(re, mach):
    """Stand-in converged interior state of (Re, Mach)."""
    x = np.linspace(0, 1, IM * JM * 5).reshape((IM, JM, 5), order="F")
    return 1.0 + 0.01 * re * x + mach * x ** 2


class FakeNewton:
    """Converges from the uniform flow (in 8 iterations) and from any other
    state within `reach` of the stand-in solution, unless its point is in
    `refuse` (iterations grow with the distance); records every start."""

    def __init__(self, reach=np.inf, refuse=()):
        self.reach, self.refuse, self.calls = reach, set(refuse), []

    def __call__(self, case, w0, tol=1e-10, maxit=12, diverge=1e3, solver=None):
        re, mach = case["phys"]["re_key"]
        gh = 3
        start = np.array(w0[gh:-gh, gh:-gh, :])
        dist = float(np.abs(start - _truth(re, mach)).max())
        uniform = bool(np.all(start == case["w"][gh:-gh, gh:-gh, :]))
        self.calls.append(dict(key=(re, mach), start=start, uniform=uniform, dist=dist))
        ok = uniform or (dist <= self.reach and (re, mach) not in self.refuse)
        it = 8 if uniform else 2 + int(np.ceil(np.log10(max(dist, 1e-12) / 1e-12)))
        rec = dict(converged=ok, iterations=it, seconds=0.01 * it, first_norm=dist, final_norm=0.0 if ok else dist,
                   norms=[dist], solves=[])
        if not ok:
            return None, rec
        w = np.array(w0, copy=True)
        w[gh:-gh, gh:-gh, :] = _truth(re, mach)
        return w, rec


@pytest.fixture
def patched(monkeypatch):
    real_case = WS.cyl_case

    def case(im, jm, mach=0.1, reynolds=47.0, noise=1e-3, ratio=1.05, **kw):
        c = real_case(im, jm, mach=mach, reynolds=reynolds, noise=noise, ratio=ratio, **kw)
        c["phys"]["re_key"] = (float(reynolds), float(mach))
        return c

    monkeypatch.setattr(WS, "cyl_case", case)
    return monkeypatch


def test_continuation_order_and_neighbour_starts(patched):
    params = np.array([[40.0, 0.05], [200.0, 0.3], [60.0, 0.07], [180.0, 0.28], [120.0, 0.15]])
    fake = FakeNewton()
    patched.setattr(WS, "newton_to_tol", fake)
    states, recs = WS.solve_baseflows(params, IM, JM)
    assert all(s is not None for s in states)
    assert recs[0]["start"] == "grid sequencing from the uniform flow" and fake.calls[0]["uniform"]
    a, b = WS.normalise(params[:, 0], params[:, 1])
    p = np.stack([a, b], 1)
    solved = [0]
    for call in fake.calls[1:]:
        u = [i for i in range(len(params)) if tuple(params[i]) == call["key"]][0]
        # the start is the state of the solved point nearest to u, and u was the
        # unsolved point nearest to the solved set
        d = np.linalg.norm(p[solved] - p[u], axis=1)
        src = solved[int(np.argmin(d))]
        assert np.array_equal(call["start"], states[src])
        unsolved = [i for i in range(len(params)) if i not in solved]
        dmin = np.linalg.norm(p[unsolved][:, None] - p[solved][None], axis=2).min(axis=1)
        assert np.isclose(dmin[unsolved.index(u)], dmin.min())
        solved.append(u)
    for i, s in enumerate(states):
        assert np.array_equal(s, _truth(*params[i]))


def test_failed_neighbour_start_retries_from_uniform(patched):
    params = np.array([[40.0, 0.05], [50.0, 0.06]])
    fake = FakeNewton(refuse=[(50.0, 0.06)])
    patched.setattr(WS, "newton_to_tol", fake)
    states, recs = WS.solve_baseflows(params, IM, JM)
    assert states[1] is not None and recs[1]["start"] == "grid sequencing after the neighbour failed"
    assert [c["uniform"] for c in fake.calls] == [True, False, True]


def fake_iterations(fake, k):
    return 2 + int(np.ceil(np.log10(max(fake.calls[k]["dist"], 1e-12) / 1e-12)))


class FakeModel:
    def __init__(self, offset):
        self.offset = offset

    def predict(self, theta, rho, re, mach):
        case = WS.cyl_case(IM, JM, mach=mach, reynolds=re, noise=0.0)
        return WS.encode(_truth(re, mach) + self.offset, case["phys"])


def test_compare_starts_plain_and_learned(patched):
    train = np.array([[40.0, 0.05], [200.0, 0.3], [100.0, 0.1]])
    states = [_truth(*p) for p in train]
    held = np.array([[110.0, 0.12]])
    fake = FakeNewton()
    patched.setattr(WS, "newton_to_tol", fake)
    out = WS.compare_starts(FakeModel(1e-6), train, states, held, IM, JM)
    r = out[0]
    # plain: the nearest training state (Re 100, Mach 0.1) as the start
    assert np.array_equal(fake.calls[0]["start"], states[2])
    assert not r["plain"]["fallback"] and not r["learned"]["fallback"]
    assert r["learned"]["first_norm"] < r["plain"]["first_norm"]
    assert r["learned"]["iterations"] < r["plain"]["iterations"]


def test_compare_starts_fallbacks(patched):
    train = np.array([[40.0, 0.05], [200.0, 0.3]])
    states = [_truth(*p) for p in train]
    held = np.array([[120.0, 0.2]])
    # neither the neighbour nor a poor guess is within reach: both arms fall back
    fake = FakeNewton(reach=0.5)
    patched.setattr(WS, "newton_to_tol", fake)
    out = WS.compare_starts(FakeModel(5.0), train, states, held, IM, JM)
    r = out[0]
    assert r["plain"]["fallback"] and r["plain"]["converged"]
    assert r["learned"]["fallback"] and r["learned"]["converged"]
    assert r["learned"]["iterations"] == fake_iterations(fake, 2) + 8  # both attempts counted
    starts = [c["uniform"] for c in fake.calls]
    assert starts == [False, True, False, True]


def test_sequence_levels():
    assert WS.sequence_levels(512, 256) == [(56, 42), (112, 84), (224, 168), (448, 256), (512, 256)]
    assert WS.sequence_levels(112, 84) == [(56, 42), (112, 84)]
    assert WS.sequence_levels(56, 42) == [(56, 42)]
    assert WS.sequence_levels(28, 21) == [(28, 21)]
    assert WS.radial_ratio(42) == 1.05 ** 0.5


def test_interpolate_state_between_o_meshes():
    """A smooth field of (azimuth, log radius) interpolated from one O-mesh of
    the family to a finer one is close to the field itself, and the identity
    on the same grid; the azimuth is periodic."""
    def field(g):
        gh = 3
        xc, yc = g["xc"][gh:-gh, gh:-gh], g["yc"][gh:-gh, gh:-gh]
        th, lr = np.arctan2(yc, xc), np.log(np.hypot(xc, yc))
        return np.stack([np.cos(th) + lr, np.sin(2 * th) * lr, lr ** 2, np.cos(th) * np.sin(th), 1.0 + 0 * lr], -1)
    from tests import helpers as H
    coarse = WS.cyl_case(56, 42, ratio=WS.radial_ratio(42), noise=0.0, ops=H.OracleOps)["grid"]
    fine = WS.cyl_case(112, 84, ratio=WS.radial_ratio(84), noise=0.0, ops=H.OracleOps)["grid"]
    fc = field(coarse)
    assert np.allclose(WS.interpolate_state(coarse, coarse, fc), fc, atol=1e-12)
    got = WS.interpolate_state(fine, coarse, fc)
    want = field(fine)
    inner = slice(1, -1)  # the last radial cells lie past the coarse centres (clamped)
    assert np.abs(got[:, inner] - want[:, inner]).max() < 0.02 * np.abs(want).max()
