"""Learned warm start of the cylinder base-flow Newton iteration.

A conditioned MLP maps (Re, Mach) and a cell's position on the O-mesh to the
converged base flow at that cell.  It is trained on base flows the solver
itself produces (broadcast_gb300.newton.CylNewton, the GPU Newton iteration
of cylinder.py:841-1068) and gives the Newton iteration its initial state for
a new (Re, Mach); the plain method it is compared with is the reference's
practice of restarting from the nearest converged neighbour
(restart_init.read_init + interpgrid, cylinder.py:560-589,
BROADCAST_npz.py:1062-1067), which is also the fallback when the learned
guess does not converge.

Network: 128 input features (the cell's azimuth as 24 harmonics, its
normalised log radius as 24 half-wave harmonics, the normalised Reynolds and
Mach numbers with 6 harmonics each, a few products), three tanh layers of
width 256, a linear output of the 5 conserved variables (padded to 128 rows
for the 128-wide tiles); every product on the tensor cores with BF16 operands
and FP32 accumulation, FP32 master weights and Adam moments
(csrc/mlp.cu).  Outputs are the conserved variables relative to the free
stream, density scaled by 1/M^2, each standardised over the training set.
Torch tensors only hold the device memory; every operation is a kernel of
libbroadcast_gb300.so.
"""
import math
import time

import numpy as np

from . import _lib
from .cases import cyl_case

RE_RANGE = (40.0, 200.0)
MACH_RANGE = (0.05, 0.3)
DIMS = (128, 256, 256, 256, 128)  # input features, three hidden layers, padded output
NOUT = 5
EPI_TANH, EPI_DTANH, EPI_LOSS = 0, 1, 2


def normalise(re, mach):
    return ((np.asarray(re, float) - RE_RANGE[0]) / (RE_RANGE[1] - RE_RANGE[0]),
            (np.asarray(mach, float) - MACH_RANGE[0]) / (MACH_RANGE[1] - MACH_RANGE[0]))


def cell_coordinates(grid):
    """Azimuth and normalised log radius of the interior cell centres, cell
    index c = i + im j (the Fortran order of the interior)."""
    gh = int(grid["gh"])
    xc = grid["xc"][gh:-gh, gh:-gh]
    yc = grid["yc"][gh:-gh, gh:-gh]
    r = np.hypot(xc, yc)
    r_in, r_out = float(r.min()), float(r.max())
    theta = np.arctan2(yc, xc)
    rho = np.log(r / r_in) / np.log(r_out / r_in)
    return (np.ravel(theta, order="F").astype(np.float32), np.ravel(rho, order="F").astype(np.float32))


def encode(w_int, phys):
    """Interior state (im, jm, 5) -> unscaled targets (ncell, 5): conserved
    variables minus the free stream, density divided by M^2."""
    t = np.reshape(w_int, (-1, 5), order="F") - np.asarray(phys["state"])[None, :]
    t = t.copy()
    t[:, 0] /= phys["mach"] ** 2
    return t


def decode(t, phys, im, jm):
    t = np.array(t, dtype=np.float64)
    t[:, 0] *= phys["mach"] ** 2
    return np.reshape(t + np.asarray(phys["state"])[None, :], (im, jm, 5), order="F")


class SurrogateMLP:
    """The network, its Adam state and its work buffers on the GPU."""

    def __init__(self, seed=0, device="cuda"):
        import torch
        _lib.load()
        self.torch, self.dev = torch, torch.device(device)
        _lib.call("bcg_set_stream", torch.cuda.current_stream(self.dev).cuda_stream)
        rng = np.random.default_rng(seed)
        f32 = dict(dtype=torch.float32, device=self.dev)
        self.w, self.b, self.mw, self.vw, self.mb, self.vb, self.wbf, self.wtbf = ([] for _ in range(8))
        for li in range(4):
            n_in, n_out = DIMS[li], DIMS[li + 1]
            live = NOUT if li == 3 else n_out
            lim = math.sqrt(6.0 / (n_in + live))  # Glorot uniform
            w = np.zeros((n_out, n_in), np.float32)
            w[:live] = rng.uniform(-lim, lim, size=(live, n_in))
            self.w.append(torch.from_numpy(w).to(self.dev))
            self.b.append(torch.zeros(n_out, **f32))
            self.mw.append(torch.zeros(n_out, n_in, **f32))
            self.vw.append(torch.zeros(n_out, n_in, **f32))
            self.mb.append(torch.zeros(n_out, **f32))
            self.vb.append(torch.zeros(n_out, **f32))
            self.wbf.append(torch.empty(n_out, n_in, dtype=torch.bfloat16, device=self.dev))
            self.wtbf.append(torch.empty(n_in, n_out, dtype=torch.bfloat16, device=self.dev))
            _lib.call("bcg_mlp_cast_weights", self.w[li], n_out, n_in, self.wbf[li], self.wtbf[li])
        self.step_count = 0
        self.scale = np.ones(NOUT)
        self._m = 0

    # -- work buffers sized for m rows
    def _buffers(self, m):
        if m == self._m:
            return
        t = self.torch
        bf = dict(dtype=t.bfloat16, device=self.dev)
        self.x = t.empty(m, DIMS[0], **bf)
        self.y = [t.empty(m, DIMS[i + 1], **bf) for i in range(3)]
        self.dz = [t.empty(m, DIMS[i + 1], **bf) for i in range(4)]
        self.t = t.empty(m, NOUT, dtype=t.float32, device=self.dev)
        self.out = t.empty(m, NOUT, dtype=t.float32, device=self.dev)
        self.lossp = t.empty((DIMS[4] // 128) * (m // 128), dtype=t.float32, device=self.dev)
        self.nsplit = max(1, min(64, m // 256))
        while m % (64 * self.nsplit):
            self.nsplit -= 1
        self.bsplit = m // 64  # column sums in chunks of 64 rows
        self.wpart = t.empty(self.nsplit * 256 * 256, dtype=t.float32, device=self.dev)
        self.bpart = t.empty(self.bsplit * 256, dtype=t.float32, device=self.dev)
        self.lsum = t.empty(1, dtype=t.float32, device=self.dev)
        self._m = m

    def forward(self, m, m_valid, target=None, out=None, gscale=0.0):
        L = _lib.call
        h = self.x
        for li in range(3):
            L("bcg_mlp_gemm_nn", EPI_TANH, h, self.wbf[li], self.b[li], None, None, self.y[li], None, None,
              m, DIMS[li + 1], DIMS[li], NOUT, m_valid, 0.0)
            h = self.y[li]
        L("bcg_mlp_gemm_nn", EPI_LOSS, h, self.wbf[3], self.b[3], None, target,
          self.dz[3] if target is not None else None, out, self.lossp if target is not None else None,
          m, DIMS[4], DIMS[3], NOUT, m_valid, gscale)

    def backward(self, m, lr, beta1=0.9, beta2=0.999, eps=1e-8, grads=None):
        """Loss gradients through the layers, weight and bias gradients, Adam
        (lr = 0: gradients only, into grads[li] if given)."""
        L = _lib.call
        for li in (3, 2, 1):
            L("bcg_mlp_gemm_nn", EPI_DTANH, self.dz[li], self.wtbf[li], None, self.y[li - 1], None,
              self.dz[li - 1], None, None, m, DIMS[li], DIMS[li + 1], NOUT, m, 0.0)
        for li in range(4):
            xin = self.x if li == 0 else self.y[li - 1]
            n1, n2 = DIMS[li + 1], DIMS[li]
            L("bcg_mlp_gemm_tn", self.dz[li], xin, self.wpart, m, n1, n2, self.nsplit)
            L("bcg_mlp_colsum", self.dz[li], m, n1, self.bsplit, self.bpart)
            L("bcg_mlp_adam", self.wpart, self.nsplit, self.bpart, self.bsplit, n1, n2, self.w[li], self.mw[li],
              self.vw[li], self.b[li], self.mb[li], self.vb[li], self.wbf[li], self.wtbf[li], float(lr), beta1, beta2,
              eps, grads[li] if grads is not None else None)

    def set_data(self, theta, rho, params, targets):
        """Training set: cell coordinates (ncell), normalised (Re, Mach) per
        base flow (nset, 2) and unscaled targets (nset, ncell, 5); the targets
        are standardised per variable here."""
        t = self.torch
        targets = np.asarray(targets, np.float64)
        sd = targets.reshape(-1, NOUT).std(axis=0)
        self.scale = np.where(sd > 0, sd, 1.0)
        self.theta = t.from_numpy(np.asarray(theta, np.float32)).to(self.dev)
        self.rho = t.from_numpy(np.asarray(rho, np.float32)).to(self.dev)
        self.params = t.from_numpy(np.asarray(params, np.float32).reshape(-1, 2).copy()).to(self.dev)
        self.targets = t.from_numpy((targets / self.scale).astype(np.float32).reshape(-1)).to(self.dev)
        self.ncell, self.nset = int(self.theta.numel()), int(self.params.shape[0])

    def fit(self, steps=3000, batch=16384, lr=2e-3, lr_final=2e-5, beta1=0.9, beta2=0.999, log_every=250, seed=7):
        """Adam on random (base flow, cell) samples, cosine step size; returns
        the logged (step, loss) pairs."""
        m = batch
        self._buffers(m)
        log = []
        gscale = 2.0 / (m * NOUT)
        for s in range(steps):
            self.step_count += 1
            k = self.step_count
            lr_s = lr_final + 0.5 * (lr - lr_final) * (1.0 + math.cos(math.pi * s / max(1, steps - 1)))
            lr_t = lr_s * math.sqrt(1.0 - beta2 ** k) / (1.0 - beta1 ** k)
            _lib.call("bcg_mlp_features", self.theta, self.rho, self.ncell, self.params, self.nset, self.targets,
                      NOUT, int(seed) * 1000003 + k, 0, m, m, self.x, self.t)
            self.forward(m, m, target=self.t, gscale=gscale)
            if log_every and (s % log_every == 0 or s == steps - 1):
                _lib.call("bcg_mlp_sum", self.lossp, int(self.lossp.numel()), self.lsum)
                log.append((s, float(self.lsum.item()) / (m * NOUT)))
            self.backward(m, lr_t, beta1, beta2)
        return log

    def predict(self, theta, rho, re, mach):
        """Unscaled targets (ncell, 5) for one (Re, Mach) on the cells given."""
        t = self.torch
        a, b = normalise(re, mach)
        ncell = len(theta)
        m = (ncell + 127) // 128 * 128
        self._buffers(m)
        th = t.from_numpy(np.asarray(theta, np.float32)).to(self.dev)
        rh = t.from_numpy(np.asarray(rho, np.float32)).to(self.dev)
        pr = t.tensor([float(a), float(b)], dtype=t.float32, device=self.dev)
        _lib.call("bcg_mlp_features", th, rh, ncell, pr, 1, None, NOUT, -1, 0, m, ncell, self.x, None)
        self.forward(m, ncell, target=None, out=self.out)
        return self.out[:ncell].cpu().numpy().astype(np.float64) * self.scale[None, :]


# ---------------------------------------------------------------------------
# base flows and the time-to-tolerance comparison

def radial_ratio(jm):
    """Radial stretching of the O-meshes here: one family of grids from r = 0.5
    to 50 D whose jm-cell member stretches by 1.05^(21/jm) per cell (1.05^0.5
    at jm = 42), so that doubling jm halves each cell; 512 x 256 has a first
    cell of 0.11 D."""
    return 1.05 ** (21.0 / jm)


def newton_to_tol(case, w0, tol=1e-10, maxit=12, diverge=1e3, solver=None):
    """Newton's iteration (CylNewton, cfl 1e10) from w0 until the max L2
    residual norm is <= tol; stops early when the norm is not finite or grows
    `diverge` times above its first value.  solver: None (the FP64 band LU)
    or a linsolve.KrylovSolver shared between calls.  Returns the state and a
    record."""
    from .newton import CylNewton
    nt = CylNewton(case, solver=solver)
    w = np.array(w0, dtype=np.float64, order="F", copy=True)
    t0 = time.perf_counter()
    n0 = None
    norms = []
    nlog = len(getattr(solver, "log", []))
    for it in range(1, maxit + 1):
        norm, dw = nt.step(w, first=(it == 1), tol=tol)
        nmax = float(np.max(norm))
        norms.append(nmax)
        n0 = nmax if n0 is None else n0
        if dw is None:
            return w, dict(converged=True, iterations=it, seconds=time.perf_counter() - t0, first_norm=n0,
                           final_norm=nmax, norms=norms, solves=getattr(solver, "log", [])[nlog:])
        if not np.isfinite(nmax) or nmax > diverge * max(n0, 1.0):
            break
    return None, dict(converged=False, iterations=it, seconds=time.perf_counter() - t0, first_norm=n0,
                      final_norm=nmax, norms=norms, solves=getattr(solver, "log", [])[nlog:])


def interpolate_state(grid_to, grid_from, w_from):
    """Interior state on O-mesh grid_from (im', jm', 5) onto grid_to: bilinear
    in the azimuth (periodic) and the logarithm of the radius of the cell
    centres; returns (im, jm, 5)."""
    def polar(g):
        gh = int(g["gh"])
        xc, yc = g["xc"][gh:-gh, gh:-gh], g["yc"][gh:-gh, gh:-gh]
        return np.arctan2(yc[:, 0], xc[:, 0]), np.log(np.hypot(xc[0, :], yc[0, :]))
    th_f, lr_f = polar(grid_from)
    th_t, lr_t = polar(grid_to)
    imf, jmf = len(th_f), len(lr_f)
    # azimuth falls with i (clockwise from the upstream point): fractional source index
    fi = np.mod((th_f[0] - th_t) / (2.0 * np.pi / imf), imf)
    i0 = np.floor(fi).astype(int)
    ai = (fi - i0)[:, None, None]
    i1 = (i0 + 1) % imf
    i0 %= imf
    fj = np.interp(lr_t, lr_f, np.arange(jmf))
    j0 = np.minimum(np.floor(fj).astype(int), jmf - 2)
    aj = (fj - j0)[None, :, None]
    j1 = j0 + 1
    W = np.asarray(w_from)
    return ((1 - ai) * ((1 - aj) * W[i0][:, j0] + aj * W[i0][:, j1]) +
            ai * ((1 - aj) * W[i1][:, j0] + aj * W[i1][:, j1]))


def sequence_levels(im, jm, coarsest=(56, 42)):
    """Grids of a sequence from the coarsest member of the family to (im, jm):
    the coarsest doubled in both directions while that stays within (im, jm),
    then steps of at most twice each extent up to (im, jm); a grid not finer
    than the coarsest is its own sequence."""
    if im <= coarsest[0] or jm <= coarsest[1]:
        return [(im, jm)]
    levels = [tuple(coarsest)]
    while 2 * levels[-1][0] <= im and 2 * levels[-1][1] <= jm:
        levels.append((2 * levels[-1][0], 2 * levels[-1][1]))
    while levels[-1] != (im, jm):
        a, b = levels[-1]
        levels.append((min(2 * a, im), min(2 * b, jm)))
    return levels


def sequenced_baseflow(re, mach, im, jm, tol=1e-10, maxit=12, solver=None, log=None):
    """A base flow without a converged neighbour: Newton's iteration from the
    uniform flow on the coarsest grid of the family (56 x 42), then on each
    finer grid of sequence_levels from the previous grid's solution
    interpolated (grid sequencing); the finest level uses `solver`, the others
    above 20000 cells a Krylov solver of their own.  Returns the finest
    level's state (or None) and a record."""
    t0 = time.perf_counter()
    prev, w_int, iters = None, None, []
    levels = sequence_levels(im, jm)
    for k, (a, b) in enumerate(levels):
        case = cyl_case(a, b, mach=float(mach), reynolds=float(re), noise=0.0, ratio=radial_ratio(b))
        w0 = case["w"] if prev is None else _full_state(case, interpolate_state(case["grid"], prev["grid"], w_int))
        if k == len(levels) - 1:
            lsolve = solver
        elif a * b > 20000:  # an intermediate level of its own size: FP64 GMRES, FP32 band LU
            from .linsolve import KrylovSolver, folded_ring_order
            lsolve = KrylovSolver(perm=folded_ring_order(a, b))
        else:
            lsolve = None
        w, rec = newton_to_tol(case, w0, tol=tol, maxit=maxit, solver=lsolve)
        iters.append(rec["iterations"])
        if log:
            log("  sequence level %dx%d: %s in %d iterations, %.1f s, norms %s%s" % (
                a, b, "converged" if w is not None else "FAILED", rec["iterations"], rec["seconds"],
                " ".join("%.1e" % x for x in rec["norms"]),
                "" if not rec["solves"] else "; GMRES iterations %s, factorisations %d" % (
                    [k["iterations"] for k in rec["solves"]], sum(k["refactored"] for k in rec["solves"]))))
        if w is None:
            return None, dict(converged=False, iterations=sum(iters), seconds=time.perf_counter() - t0,
                              first_norm=rec["first_norm"], final_norm=rec["final_norm"], levels=levels)
        gh = int(case["grid"]["gh"])
        prev, w_int = case, w[gh:-gh, gh:-gh, :].copy(order="F")
    return w, dict(converged=True, iterations=sum(iters), seconds=time.perf_counter() - t0, first_norm=None,
                   final_norm=None, levels=levels, level_iterations=iters)


def _full_state(case, w_int):
    gh = int(case["grid"]["gh"])
    w = case["w"].copy(order="F")
    w[gh:-gh, gh:-gh, :] = w_int
    return w


def sample_parameters(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(*RE_RANGE, size=n), rng.uniform(*MACH_RANGE, size=n)], axis=1)


def solve_baseflows(params, im, jm, ratio=None, tol=1e-10, maxit=12, log=None, solver=None):
    """Converged base flows at every (Re, Mach) of params by continuation:
    the first by grid sequencing from the uniform flow on the coarsest grid
    of the family, each next one (the unsolved point nearest to a solved one)
    from its nearest solved neighbour, retried by grid sequencing if that does
    not converge.  solver: the linear solve of the (im, jm) Newton iterations
    (None: the FP64 band LU; a linsolve.KrylovSolver is shared by all of them,
    its FP32 factor reused from one base flow to the next).  Returns the
    interior states (None where both failed) and the per-point records."""
    ratio = radial_ratio(jm) if ratio is None else ratio
    n = len(params)
    a, b = normalise(params[:, 0], params[:, 1])
    p = np.stack([a, b], axis=1)
    states, recs = [None] * n, [None] * n
    solved = []
    todo = list(range(n))
    while todo:
        if not solved:
            u, src = todo[0], None
        else:
            d = np.linalg.norm(p[todo][:, None, :] - p[solved][None, :, :], axis=2)
            iu, isv = np.unravel_index(np.argmin(d), d.shape)
            u, src = todo[iu], solved[isv]
        todo.remove(u)
        case = cyl_case(im, jm, mach=float(params[u, 1]), reynolds=float(params[u, 0]), noise=0.0, ratio=ratio)
        gh = int(case["grid"]["gh"])
        if src is None:
            w, rec = sequenced_baseflow(params[u, 0], params[u, 1], im, jm, tol=tol, maxit=maxit, solver=solver, log=log)
            rec["start"] = "grid sequencing from the uniform flow"
        else:
            w, rec = newton_to_tol(case, _full_state(case, states[src]), tol=tol, maxit=maxit, solver=solver)
            rec["start"] = "neighbour"
            if w is None:
                w, rec2 = sequenced_baseflow(params[u, 0], params[u, 1], im, jm, tol=tol, maxit=maxit, solver=solver,
                                             log=log)
                rec2["start"] = "grid sequencing after the neighbour failed"
                rec2["seconds"] += rec["seconds"]
                rec = rec2
        recs[u] = rec
        if w is not None:
            states[u] = w[gh:-gh, gh:-gh, :].copy(order="F")
            solved.append(u)
        if log:
            log("base flow %d/%d Re %.1f M %.3f: %s, %d iterations, %.2f s" % (
                n - len(todo), n, params[u, 0], params[u, 1], "converged" if w is not None else "FAILED",
                rec["iterations"], rec["seconds"]))
    return states, recs


def compare_starts(model, train_params, train_states, held_params, im, jm, ratio=None, tol=1e-10, maxit=12,
                   log=None, solver=None, solver_learned=None):
    """Time to tol for every held-out (Re, Mach): from the nearest training
    base flow (plain continuation) and from the network's guess (with the
    plain start as fallback).  Each arm solves with its own linear solver
    (`solver` for the plain arm, `solver_learned` for the learned one; the same
    object when that is None), so that a solver that keeps state between solves
    (the Krylov solver's preconditioner factor) gives neither arm the other's
    work: give two solvers in the same state.  Returns per-point records."""
    solver_learned = solver if solver_learned is None else solver_learned
    ratio = radial_ratio(jm) if ratio is None else ratio
    ok = [i for i, s in enumerate(train_states) if s is not None]
    ta, tb = normalise(train_params[ok, 0], train_params[ok, 1])
    tp = np.stack([ta, tb], axis=1)
    out = []
    for re, mach in held_params:
        case = cyl_case(im, jm, mach=float(mach), reynolds=float(re), noise=0.0, ratio=ratio)
        theta, rho = cell_coordinates(case["grid"])
        a, b = normalise(re, mach)
        nn = ok[int(np.argmin(np.linalg.norm(tp - np.array([a, b])[None, :], axis=1)))]
        t0 = time.perf_counter()
        w_plain0 = _full_state(case, train_states[nn])
        _, plain = newton_to_tol(case, w_plain0, tol=tol, maxit=maxit, solver=solver)
        plain["fallback"] = False
        if not plain["converged"]:  # as the base-flow generation: grid sequencing
            _, fb = sequenced_baseflow(re, mach, im, jm, tol=tol, maxit=maxit, solver=solver)
            plain.update(fallback=True, converged=fb["converged"], iterations=plain["iterations"] + fb["iterations"])
        plain["seconds"] = time.perf_counter() - t0
        t0 = time.perf_counter()
        guess = decode(model.predict(theta, rho, re, mach), case["phys"], im, jm)
        t_guess = time.perf_counter() - t0
        _, learned = newton_to_tol(case, _full_state(case, guess), tol=tol, maxit=maxit, solver=solver_learned)
        learned["seconds"] += t_guess
        learned["guess_seconds"] = t_guess
        learned["fallback"] = False
        if not learned["converged"]:  # the plain start as fallback
            if plain["iterations"] and not plain["fallback"]:
                _, fb = newton_to_tol(case, w_plain0, tol=tol, maxit=maxit, solver=solver_learned)
            else:
                _, fb = sequenced_baseflow(re, mach, im, jm, tol=tol, maxit=maxit, solver=solver_learned)
            learned.update(fallback=True, converged=fb["converged"], seconds=learned["seconds"] + fb["seconds"],
                           iterations=learned["iterations"] + fb["iterations"])
        rec = dict(re=float(re), mach=float(mach), plain=plain, learned=learned)
        out.append(rec)
        if log:
            log("held-out Re %.1f M %.3f: plain %d it %.2f s (|R0| %.1e)%s, learned %d it %.2f s (|R0| %.1e)%s" % (
                re, mach, plain["iterations"], plain["seconds"], plain["first_norm"],
                " (fallback)" if plain["fallback"] else "", learned["iterations"], learned["seconds"],
                learned["first_norm"], " (fallback)" if learned["fallback"] else ""))
    return out


def train_on_baseflows(train_params, train_states, im, jm, ratio=None, seed=0, **fit_kw):
    """Network trained on the converged base flows (None entries skipped)."""
    ratio = radial_ratio(jm) if ratio is None else ratio
    ok = [i for i, s in enumerate(train_states) if s is not None]
    case = cyl_case(im, jm, noise=0.0, ratio=ratio)
    theta, rho = cell_coordinates(case["grid"])
    targets = []
    for i in ok:
        ph = cyl_case(im, jm, mach=float(train_params[i, 1]), reynolds=float(train_params[i, 0]), noise=0.0,
                      ratio=ratio)["phys"]
        targets.append(encode(train_states[i], ph))
    a, b = normalise(train_params[ok, 0], train_params[ok, 1])
    model = SurrogateMLP(seed=seed)
    model.set_data(theta, rho, np.stack([a, b], axis=1), np.stack(targets))
    log = model.fit(**fit_kw)
    return model, log
