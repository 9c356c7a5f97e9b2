"""CPU checks of the learned warm start's host side and of the oracle that
checks its kernels: bfloat16 rounding, the backward formulas against central
finite differences, the Adam update, the target encoding."""
import numpy as np
import pytest

from oracle import mlp_oracle as MO


def test_bf16_round_to_nearest_even():
    one = np.float32(1.0)
    vals = np.array([1.0, 1 + 2.0 ** -8, 1 + 2.0 ** -8 + 2.0 ** -20, 1 + 3 * 2.0 ** -8, -2.5, 3.0e38], np.float32)
    got = MO.bf16(vals)
    assert got[0] == one
    assert got[1] == one                       # halfway: to the even neighbour
    assert got[2] == np.float32(1 + 2.0 ** -7)  # just above halfway
    assert got[3] == np.float32(1 + 2.0 ** -6)  # halfway, odd below: up to even
    assert got[4] == np.float32(-2.5)
    assert np.all(np.abs(MO.bf16(np.linspace(-3, 3, 1001, dtype=np.float32)) - np.linspace(-3, 3, 1001)) <= 2.0 ** -7)


def _net(rng, dims):
    ws = [rng.normal(size=(dims[i + 1], dims[i])) / np.sqrt(dims[i]) for i in range(len(dims) - 1)]
    bs = [rng.normal(size=dims[i + 1]) * 0.1 for i in range(len(dims) - 1)]
    return ws, bs


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    dims = (6, 5, 4, 4, 3)
    ws, bs = _net(rng, dims)
    x = rng.normal(size=(9, dims[0]))
    t = rng.normal(size=(9, 3))
    loss, gw, gb = MO.loss_and_grads(x, t, ws, bs, nout=2, m_valid=7, exact=True)
    h = 1e-6
    for li in range(4):
        for idx in [(0, 0), (dims[li + 1] - 1, dims[li] - 1), (1, 2)]:
            wp = [w.copy() for w in ws]
            wm = [w.copy() for w in ws]
            wp[li][idx] += h
            wm[li][idx] -= h
            fd = (MO.loss_and_grads(x, t, wp, bs, 2, 7, exact=True)[0] - MO.loss_and_grads(x, t, wm, bs, 2, 7, exact=True)[0]) / (2 * h)
            assert abs(fd - gw[li][idx]) <= 1e-7 * max(1.0, abs(fd)), (li, idx, fd, gw[li][idx])
        bp = [b.copy() for b in bs]
        bm = [b.copy() for b in bs]
        bp[li][0] += h
        bm[li][0] -= h
        fd = (MO.loss_and_grads(x, t, ws, bp, 2, 7, exact=True)[0] - MO.loss_and_grads(x, t, ws, bm, 2, 7, exact=True)[0]) / (2 * h)
        assert abs(fd - gb[li][0]) <= 1e-7 * max(1.0, abs(fd))
    # the rounded (kernel-faithful) gradients stay close to the exact ones
    _, gw2, _ = MO.loss_and_grads(x, t, ws, bs, nout=2, m_valid=7)
    for a, b in zip(gw, gw2):
        assert np.abs(a - b).max() <= 0.02 * np.abs(a).max()


def test_adam_folded_bias_correction():
    rng = np.random.default_rng(1)
    w = rng.normal(size=50).astype(np.float32)
    m = np.zeros(50, np.float32)
    v = np.zeros(50, np.float32)
    w_ref, m_ref, v_ref = w.astype(np.float64), np.zeros(50), np.zeros(50)
    for step in range(1, 6):
        g = rng.normal(size=50)
        MO.adam(w, m, v, g, step, lr=1e-2, eps=0.0)
        m_ref = 0.9 * m_ref + 0.1 * g
        v_ref = 0.999 * v_ref + 0.001 * g * g
        w_ref = w_ref - 1e-2 * (m_ref / (1 - 0.9 ** step)) / np.sqrt(v_ref / (1 - 0.999 ** step))
    assert np.abs(w - w_ref).max() <= 1e-5


def test_features_layout():
    f = MO.features(np.array([0.3]), np.array([0.25]), np.array([0.5]), np.array([0.75]))
    assert f.shape == (1, 128)
    assert f[0, 0] == 1 and f[0, 1] == np.float32(0.25) and f[0, 2] == np.float32(0.5)
    assert abs(f[0, 4] - np.sin(0.3)) <= 2 ** -8 and abs(f[0, 5] - np.cos(0.3)) <= 2 ** -8
    assert abs(f[0, 53] - np.cos(np.pi * 0.25)) <= 2 ** -8
    assert abs(f[0, 102] - np.sin(np.pi * 0.75)) <= 2 ** -8
    assert f[0, 127] == 0


def test_target_encoding_roundtrip_and_coordinates():
    from broadcast_gb300 import warmstart as WS
    from broadcast_gb300.cases import cyl_case
    c = cyl_case(28, 21, mach=0.2, reynolds=80.0, noise=1e-3, ratio=1.05 ** 0.5)
    w_int = c["w"][3:-3, 3:-3, :]
    t = WS.encode(w_int, c["phys"])
    assert t.shape == (28 * 21, 5)
    assert np.abs(t[:, 1:]).max() <= 1.5e-3 and np.abs(t[:, 0]).max() <= 1.5e-3 / 0.04
    back = WS.decode(t, c["phys"], 28, 21)
    assert np.abs(back - w_int).max() <= 1e-12 * np.abs(w_int).max()
    theta, rho = WS.cell_coordinates(c["grid"])
    assert theta.shape == (28 * 21,) and rho.min() == 0 and abs(rho.max() - 1) < 1e-6
    assert np.all(np.diff(np.reshape(rho, (28, 21), order="F")[0]) > 0)  # radius grows with j
    a, b = WS.normalise(np.array([40, 200]), np.array([0.05, 0.3]))
    assert np.allclose(a, [0, 1]) and np.allclose(b, [0, 1])
