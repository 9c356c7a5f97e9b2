"""Oracle of the learned warm start's network: numpy restatement of the
conditioned MLP the CUDA kernels train and run (broadcast_gb300/csrc/mlp.cu).

Test infrastructure only: imported by tests/ as the checker of the kernels,
never by the package.  The reference (BROADCAST) has no network; the
algorithms restated here are the published ones:
  - a fully connected network y = W4 tanh(W3 tanh(W2 tanh(W1 x + b1) + b2)
    + b3) + b4 with a mean-squared-error loss and its gradient by the chain
    rule (backpropagation, Rumelhart, Hinton, Williams 1986);
  - Adam (Kingma, Ba 2015, Algorithm 1) with the bias corrections folded into
    the step size;
  - round-to-nearest-even of float32 to bfloat16 (the top 16 bits of the
    float32 pattern after adding 0x7FFF plus the kept part's lowest bit).
The kernels compute every product on bfloat16 operands with float32
accumulation and store activations and loss gradients in bfloat16; the oracle
rounds at the same points and accumulates in float64, so the two differ only
by the accumulation order (and the rare bfloat16 rounding that order flips).
"""
import numpy as np

NFEAT = 128


def bf16(x):
    """Round float32 values to bfloat16 (returned as float32), nearest-even."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).reshape(np.shape(x))


def features(theta, rho, a, b):
    """Input features of samples (arrays of equal length), float32 then
    bfloat16, in the kernel's order: 1, rho, a, b; sin/cos(k theta) k=1..24;
    sin/cos(pi k rho) k=1..24; sin/cos(pi k a), sin/cos(pi k b) k=1..6; a b,
    rho a, rho b, 0."""
    theta, rho, a, b = (np.asarray(v, dtype=np.float32) for v in (theta, rho, a, b))
    n = theta.shape[0]
    f = np.zeros((n, NFEAT), np.float32)
    pi = np.float32(3.14159265358979)
    f[:, 0], f[:, 1], f[:, 2], f[:, 3] = 1.0, rho, a, b
    for k in range(1, 25):
        kt = np.float32(k) * theta
        f[:, 4 + 2 * (k - 1)], f[:, 5 + 2 * (k - 1)] = np.sin(kt), np.cos(kt)
        kr = pi * np.float32(k) * rho
        f[:, 52 + 2 * (k - 1)], f[:, 53 + 2 * (k - 1)] = np.sin(kr), np.cos(kr)
    for k in range(1, 7):
        ka, kb = pi * np.float32(k) * a, pi * np.float32(k) * b
        f[:, 100 + 4 * (k - 1)], f[:, 101 + 4 * (k - 1)] = np.sin(ka), np.cos(ka)
        f[:, 102 + 4 * (k - 1)], f[:, 103 + 4 * (k - 1)] = np.sin(kb), np.cos(kb)
    f[:, 124], f[:, 125], f[:, 126] = a * b, rho * a, rho * b
    return bf16(f)


def _store(x, exact):
    """A value the kernels store in bfloat16 (exact: kept in float64)."""
    return x if exact else bf16(np.asarray(x, dtype=np.float32)).astype(np.float64)


def forward(x, ws, bs, exact=False):
    """Activations of every layer: [x, y1, y2, y3, z4] (float64 arrays); ws
    are the weight matrices (out x in), bs the biases.  Hidden activations are
    stored in bfloat16 as the kernels do (exact: not rounded); the output z4
    is float32 (exact: float64)."""
    acts = [np.asarray(x, dtype=np.float64)]
    h = acts[0]
    for li, (w, b) in enumerate(zip(ws, bs)):
        z = h @ np.asarray(w, np.float64).T + np.asarray(b, np.float64)
        if li < len(ws) - 1:
            h = _store(np.tanh(z), exact)
        else:
            h = z if exact else z.astype(np.float32).astype(np.float64)
        acts.append(h)
    return acts


def loss_and_grads(x, t, ws, bs, nout, m_valid=None, exact=False):
    """Mean squared error over the first m_valid rows and the first nout
    outputs, and its gradient w.r.t. every weight and bias, with the loss
    gradients stored in bfloat16 between layers as the kernels do (exact:
    float64 throughout, for finite-difference checks)."""
    m = x.shape[0] if m_valid is None else m_valid
    acts = forward(x, ws, bs, exact)
    z = acts[-1]
    d = np.zeros_like(z)
    d[:m, :nout] = z[:m, :nout] - np.asarray(t, np.float64)[:m, :nout]
    if not exact:
        d = d.astype(np.float32).astype(np.float64)
    loss = float(np.sum(d[:m, :nout] ** 2) / (m * nout))
    gscale = 2.0 / (m * nout)
    dz = _store(gscale * d, exact)
    gw, gb = [None] * len(ws), [None] * len(ws)
    for li in range(len(ws) - 1, -1, -1):
        gw[li] = dz.T @ acts[li]
        gb[li] = dz.sum(axis=0)
        if li > 0:
            y = acts[li]
            back = dz @ np.asarray(ws[li], np.float64)
            if not exact:
                back = back.astype(np.float32).astype(np.float64)
            dz = _store(back * (1.0 - y * y), exact)
    return loss, gw, gb


def adam(w, m, v, g, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (in place on float32 arrays) with the bias-corrected
    step lr sqrt(1 - beta2^t) / (1 - beta1^t)."""
    lr_t = np.float32(lr * np.sqrt(1.0 - beta2 ** step) / (1.0 - beta1 ** step))
    m[...] = np.float32(beta1) * m + np.float32(1.0 - beta1) * g.astype(np.float32)
    v[...] = np.float32(beta2) * v + np.float32(1.0 - beta2) * g.astype(np.float32) ** 2
    w[...] = w - lr_t * m / (np.sqrt(v) + np.float32(eps))
    return lr_t
