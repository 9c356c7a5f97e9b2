"""GPU checks of the learned warm start: each MLP kernel against the numpy
oracle (oracle/mlp_oracle.py), one training step's gradients, a training run,
and the warm start against the plain continuation on a small cylinder.

Tolerances: products take bfloat16 operands with float32 accumulation on
both sides of a comparison, but the kernels accumulate in a different order
than the oracle, so a stored bfloat16 value may round to its neighbour:
outputs are compared within 2 bfloat16 ulps (2^-6 relative) of the largest
value, float32 sums within 1e-5 relative."""
import numpy as np
import pytest

from oracle import mlp_oracle as MO

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _lib():
    from broadcast_gb300 import _lib
    _lib.load()
    _lib.call("bcg_set_stream", torch.cuda.current_stream().cuda_stream)
    return _lib


def _bf(a):
    return torch.from_numpy(np.asarray(a, np.float32)).cuda().to(torch.bfloat16)


def _np(t):
    return t.float().cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("epi", [0, 1, 2])
def test_gemm_nn_matches_oracle(epi):
    L = _lib()
    rng = np.random.default_rng(epi)
    m, n, k, nout, m_valid = 256, 256, 192, 5, 250
    a = MO.bf16(rng.normal(size=(m, k)).astype(np.float32))
    b = MO.bf16((rng.normal(size=(n, k)) / np.sqrt(k)).astype(np.float32))
    bias = rng.normal(size=n).astype(np.float32)
    yprev = MO.bf16(np.tanh(rng.normal(size=(m, n))).astype(np.float32))
    target = rng.normal(size=(m, nout)).astype(np.float32)
    c = a.astype(np.float64) @ b.astype(np.float64).T + bias
    out_bf = torch.zeros(m, n, dtype=torch.bfloat16, device="cuda")
    out_f = torch.zeros(m, nout, dtype=torch.float32, device="cuda")
    lossp = torch.zeros((n // 128) * (m // 128), dtype=torch.float32, device="cuda")
    tt = torch.from_numpy(target).cuda()
    bt = torch.from_numpy(bias).cuda()
    gscale = 2.0 / (m_valid * nout)
    L.call("bcg_mlp_gemm_nn", epi, _bf(a), _bf(b), bt, _bf(yprev), tt if epi == 2 else None, out_bf,
           out_f if epi == 2 else None, lossp if epi == 2 else None, m, n, k, nout, m_valid, gscale)
    torch.cuda.synchronize()
    got = _np(out_bf)
    if epi == 0:
        ref = np.tanh(c)
    elif epi == 1:
        ref = c * (1.0 - yprev.astype(np.float64) ** 2)
    else:
        d = np.zeros((m, n))
        d[:m_valid, :nout] = c[:m_valid, :nout] - target[:m_valid]
        ref = gscale * d
        assert np.abs(out_f.cpu().numpy() - c[:, :nout]).max() <= 1e-5 * np.abs(c).max()
        assert abs(lossp.sum().item() - np.sum(d ** 2)) <= 1e-5 * np.sum(d ** 2)
        assert np.all(got[m_valid:] == 0) and np.all(got[:, nout:] == 0)
    assert np.abs(got - ref).max() <= 2.0 ** -6 * np.abs(ref).max()


def test_gemm_tn_and_colsum_match_oracle():
    L = _lib()
    rng = np.random.default_rng(5)
    m, n1, n2, nsplit = 1024, 128, 256, 4
    dz = MO.bf16(rng.normal(size=(m, n1)).astype(np.float32))
    x = MO.bf16(rng.normal(size=(m, n2)).astype(np.float32))
    part = torch.zeros(nsplit * n1 * n2, dtype=torch.float32, device="cuda")
    L.call("bcg_mlp_gemm_tn", _bf(dz), _bf(x), part, m, n1, n2, nsplit)
    bpart = torch.zeros(nsplit * n1, dtype=torch.float32, device="cuda")
    L.call("bcg_mlp_colsum", _bf(dz), m, n1, nsplit, bpart)
    torch.cuda.synchronize()
    got = part.cpu().numpy().reshape(nsplit, n1, n2).astype(np.float64).sum(axis=0)
    ref = dz.astype(np.float64).T @ x.astype(np.float64)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    gb = bpart.cpu().numpy().reshape(nsplit, n1).sum(axis=0)
    assert np.abs(gb - dz.astype(np.float64).sum(axis=0)).max() <= 1e-5 * np.abs(dz).sum(axis=0).max()


def test_bad_extents_are_rejected():
    from broadcast_gb300._lib import BroadcastError
    L = _lib()
    a = torch.zeros(100, 64, dtype=torch.bfloat16, device="cuda")
    with pytest.raises(BroadcastError):
        L.call("bcg_mlp_gemm_nn", 0, a, a, None, None, None, a, None, None, 100, 128, 64, 5, 100, 0.0)
    with pytest.raises(BroadcastError):
        L.call("bcg_mlp_gemm_tn", a, a, a, 100, 128, 128, 1)
    host = np.zeros((128, 64), np.uint16)
    with pytest.raises(BroadcastError):
        L.call("bcg_mlp_gemm_nn", 0, host, host, None, None, None, host, None, None, 128, 128, 64, 5, 128, 0.0)


def test_features_match_oracle():
    L = _lib()
    rng = np.random.default_rng(3)
    ncell, nset, m = 300, 4, 384
    theta = rng.uniform(-np.pi, np.pi, ncell).astype(np.float32)
    rho = rng.uniform(0, 1, ncell).astype(np.float32)
    params = rng.uniform(0, 1, (nset, 2)).astype(np.float32)
    x = torch.empty(m, 128, dtype=torch.bfloat16, device="cuda")
    th, rh, pr = (torch.from_numpy(v).cuda() for v in (theta, rho, params))
    # inference rows: cell r of set 2
    L.call("bcg_mlp_features", th, rh, ncell, pr, nset, None, 5, -1, 2, m, ncell, x, None)
    torch.cuda.synchronize()
    ref = MO.features(theta, rho, np.full(ncell, params[2, 0]), np.full(ncell, params[2, 1]))
    got = _np(x)
    assert np.abs(got[:ncell] - ref).max() <= 2.0 ** -7 * 1.5
    assert np.all(got[ncell:] == 0)
    # training rows: each row's gathered target names its (set, cell)
    tg = np.zeros((nset, ncell, 5), np.float32)
    tg[:, :, 0] = np.arange(nset)[:, None]
    tg[:, :, 1] = np.arange(ncell)[None, :]
    t = torch.empty(m, 5, dtype=torch.float32, device="cuda")
    L.call("bcg_mlp_features", th, rh, ncell, pr, nset, torch.from_numpy(tg.ravel()).cuda(), 5, 12345, 0, m, m, x,
           t)
    torch.cuda.synchronize()
    tt = t.cpu().numpy()
    s, c = tt[:, 0].astype(int), tt[:, 1].astype(int)
    assert len(set(zip(s, c))) > m // 2  # spread over the samples
    ref = MO.features(theta[c], rho[c], params[s, 0], params[s, 1])
    assert np.abs(_np(x) - ref).max() <= 2.0 ** -7 * 1.5


def _model_and_batch(m=256, seed=0):
    from broadcast_gb300.warmstart import SurrogateMLP
    model = SurrogateMLP(seed=seed)
    rng = np.random.default_rng(seed + 10)
    # perturb the (zero-initialised) biases and the padded output rows stay zero
    for li in range(4):
        model.b[li].copy_(torch.from_numpy((0.1 * rng.normal(size=model.b[li].numel())).astype(np.float32)))
    model.b[3][5:] = 0
    model._buffers(m)
    x = MO.bf16(rng.uniform(-1, 1, size=(m, 128)).astype(np.float32))
    t = rng.normal(size=(m, 5)).astype(np.float32)
    model.x.copy_(_bf(x))
    model.t.copy_(torch.from_numpy(t).cuda())
    return model, x, t


def _oracle_weights(model):
    ws = [_np(w) for w in model.wbf]
    bs = [b.cpu().numpy().astype(np.float64) for b in model.b]
    return ws, bs


def test_training_step_gradients_match_oracle():
    """One forward and backward pass (lr = 0: gradients only) against the
    oracle's chain rule on the same bfloat16 weights and inputs."""
    m, m_valid = 256, 250
    model, x, t = _model_and_batch(m)
    ws, bs = _oracle_weights(model)
    loss, gw, gb = MO.loss_and_grads(x, t, ws, bs, nout=5, m_valid=m_valid)
    grads = [torch.zeros(model.w[li].numel() + model.b[li].numel(), dtype=torch.float32, device="cuda")
             for li in range(4)]
    model.forward(m, m_valid, target=model.t, gscale=2.0 / (m_valid * 5))
    model.backward(m, 0.0, grads=grads)
    _lib().call("bcg_mlp_sum", model.lossp, int(model.lossp.numel()), model.lsum)
    torch.cuda.synchronize()
    assert abs(model.lsum.item() / (m_valid * 5) - loss) <= 1e-3 * loss
    for li in range(4):
        g = grads[li].cpu().numpy().astype(np.float64)
        n1, n2 = model.w[li].shape
        gwk, gbk = g[:n1 * n2].reshape(n1, n2), g[n1 * n2:]
        scale = np.abs(gw[li]).max()
        assert np.abs(gwk - gw[li]).max() <= 2e-2 * scale, (li, np.abs(gwk - gw[li]).max(), scale)
        assert np.abs(gbk - gb[li]).max() <= 2e-2 * np.abs(gb[li]).max()
    # the padded output rows get no gradient
    assert np.all(grads[3].cpu().numpy()[: 128 * 256].reshape(128, 256)[5:] == 0)


def test_adam_step_matches_oracle():
    m = 256
    model, x, t = _model_and_batch(m, seed=1)
    w0 = [w.cpu().numpy().copy() for w in model.w]
    b0 = [b.cpu().numpy().copy() for b in model.b]
    grads = [torch.zeros(model.w[li].numel() + model.b[li].numel(), dtype=torch.float32, device="cuda")
             for li in range(4)]
    model.forward(m, m, target=model.t, gscale=2.0 / (m * 5))
    lr = 1e-3
    lr_t = lr * np.sqrt(1 - 0.999) / (1 - 0.9)
    model.backward(m, lr_t, grads=grads)
    torch.cuda.synchronize()
    for li in range(4):
        g = grads[li].cpu().numpy()
        n1, n2 = w0[li].shape
        w, mm, vv = w0[li].ravel().copy(), np.zeros(n1 * n2, np.float32), np.zeros(n1 * n2, np.float32)
        MO.adam(w, mm, vv, g[:n1 * n2], 1, lr)
        assert np.abs(model.w[li].cpu().numpy().ravel() - w).max() <= 1e-6
        b, mb, vb = b0[li].copy(), np.zeros(n1, np.float32), np.zeros(n1, np.float32)
        MO.adam(b, mb, vb, g[n1 * n2:], 1, lr)
        assert np.abs(model.b[li].cpu().numpy() - b).max() <= 1e-6
        assert np.all(_np(model.wbf[li]) == MO.bf16(model.w[li].cpu().numpy()))
        assert np.all(_np(model.wtbf[li]) == _np(model.wbf[li]).T)


def test_training_fits_a_smooth_field():
    """The network learns a smooth field of (theta, rho, a, b) on the GPU:
    the loss falls by more than 30x in 400 Adam steps."""
    from broadcast_gb300.warmstart import SurrogateMLP
    rng = np.random.default_rng(4)
    ncell, nset = 600, 12
    theta = rng.uniform(-np.pi, np.pi, ncell)
    rho = rng.uniform(0, 1, ncell)
    params = rng.uniform(0, 1, (nset, 2))
    f = lambda th, r, a, b: np.stack([np.sin(th) * r + a, np.cos(2 * th) * b, r * r - a * b, 0 * r, np.exp(-3 * r) * (1 + a)], -1)
    targets = np.stack([f(theta, rho, p[0], p[1]) for p in params])
    model = SurrogateMLP(seed=0)
    model.set_data(theta, rho, params, targets)
    log = model.fit(steps=400, batch=4096, lr=2e-3, log_every=100)
    assert log[-1][1] < log[0][1] / 30, log
    pred = model.predict(theta, rho, 40 + 160 * params[3, 0], 0.05 + 0.25 * params[3, 1])
    assert np.abs(pred - targets[3]).max() <= 0.1 * np.abs(targets).max()


def test_warm_start_against_plain_continuation():
    """Cylinder 28 x 21: base flows at 12 (Re, Mach) points by continuation,
    the network trained on them, then 2 held-out points solved to 1e-10 from
    the network's guess and from the nearest neighbour (plain continuation,
    restarted from the uniform flow if it does not converge); the guess must
    converge by itself, start closer to the solution (smaller first residual)
    and need no more Newton iterations than the plain start."""
    from broadcast_gb300 import warmstart as WS
    im, jm, ratio = 28, 21, 1.05
    train = WS.sample_parameters(12, seed=5)
    states, recs = WS.solve_baseflows(train, im, jm, ratio=ratio)
    assert all(s is not None for s in states), recs
    model, log = WS.train_on_baseflows(train, states, im, jm, ratio=ratio, steps=600, batch=4096, log_every=200)
    assert log[-1][1] < log[0][1] / 30
    held = WS.sample_parameters(2, seed=6)
    out = WS.compare_starts(model, train, states, held, im, jm, ratio=ratio)
    for r in out:
        assert r["plain"]["converged"] and r["learned"]["converged"], r
        assert not r["learned"]["fallback"], r
        assert r["learned"]["first_norm"] < r["plain"]["first_norm"], r
        assert r["learned"]["iterations"] <= r["plain"]["iterations"], r
