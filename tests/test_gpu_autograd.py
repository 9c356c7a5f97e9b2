"""The residual, its tangent and its adjoint behind torch.autograd.Function
(broadcast_gb300.autograd), on the 256x256 cylinder O-mesh (Mach 0.1, Re 47,
uniform flow + 1e-3 noise, seed 1) with 32 seeded Gaussian directions on the
interior (seed 2):

  forward mode  : against central finite differences of the GPU residual,
                  h = 1e-7, tolerance 1e-6 of the largest |R'(w) v| per
                  variable (rounding of R at h = 1e-7 is ~1e-9 of it, the
                  truncation ~1e-14), and against the oracle's tangent (the
                  restatement pinned to Tapenade's flux_num_dnc5_d) at 1e-11;
  reverse mode  : against the oracle's adjoint (pinned to flux_num_dnc5_b) at
                  1e-11 and the dot-product identity <R'v, u> = <v, R'^T u>.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu
NDIR = 32
H_FD = 1e-7


@pytest.fixture(scope="module")
def setup():
    import torch
    from broadcast_gb300.operator import Dnc5Operator, to_device
    c = H.cyl_case(256, 256, seed=1)
    H.oracle_bcs(c, c["w"])
    op = Dnc5Operator(c["grid"], c["phys"])
    rng = np.random.default_rng(2)
    v = np.zeros((NDIR,) + c["w"].shape)
    v[:, 3:-3, 3:-3, :] = rng.standard_normal((NDIR, 256, 256, 5))
    w = to_device(c["w"])
    vt = torch.stack([to_device(np.asfortranarray(x)) for x in v])
    return c, op, w, v, vt


def _scale(a):
    return np.maximum(np.abs(H.interior(a)).reshape(-1, 5).max(0), 1e-300)


def test_forward_value(setup):
    from broadcast_gb300.autograd import residual
    from broadcast_gb300.operator import to_host
    c, op, w, _, _ = setup
    r = to_host(residual(w, op))
    ref = O.residual(c["grid"], c["phys"], c["w"])
    assert H.rel_err(r, ref, H.flux_scale(c, c["w"])) < 1e-12


def test_forward_mode_against_fd_and_oracle(setup):
    import torch
    import torch.autograd.forward_ad as fwAD
    from broadcast_gb300.autograd import residual
    from broadcast_gb300.operator import to_host
    c, op, w, v, vt = setup
    jv = []
    for k in range(NDIR):
        with fwAD.dual_level():
            out = residual(fwAD.make_dual(w, vt[k]), op)
            jv.append(to_host(fwAD.unpack_dual(out).tangent.clone()))
    torch.cuda.synchronize()
    # finite differences of the GPU residual
    for k in range(NDIR):
        rp = to_host(op.residual(w + H_FD * vt[k]).clone())
        rm = to_host(op.residual(w - H_FD * vt[k]).clone())
        fd = (rp - rm) / (2.0 * H_FD)
        err = (np.abs(H.interior(fd - jv[k])).reshape(-1, 5).max(0) / _scale(jv[k])).max()
        assert err < 1e-6, (k, err)
    # the oracle's tangent on all 32 directions
    _, ref = O.jvp(c["grid"], c["phys"], c["w"], v)
    for k in range(NDIR):
        err = (np.abs(H.interior(jv[k] - ref[k])).reshape(-1, 5).max(0) / _scale(ref[k])).max()
        assert err < 1e-11, (k, err)


def test_reverse_mode_against_oracle_and_dot_product(setup):
    import torch
    from broadcast_gb300.autograd import residual
    from broadcast_gb300.operator import to_device, to_host
    c, op, w, v, vt = setup
    rng = np.random.default_rng(3)
    u = np.zeros_like(c["w"])
    u[3:-3, 3:-3] = rng.standard_normal((256, 256, 5))
    wr = w.clone().requires_grad_(True)
    (g,) = torch.autograd.grad(residual(wr, op), wr, grad_outputs=to_device(u))
    wb = to_host(g)
    ref = O.vjp(c["grid"], c["phys"], c["w"], u)
    sc = np.abs(ref).reshape(-1, 5).max(0)
    assert (np.abs(wb - ref).reshape(-1, 5).max(0) / sc).max() < 1e-11
    _, jv = op.jvp(w, vt)
    jv = jv.cpu().numpy()
    ut = to_device(u).cpu().numpy()
    for k in range(NDIR):
        lhs = float(np.vdot(jv[k], ut))
        rhs = float(np.vdot(vt[k].cpu().numpy(), g.cpu().numpy()))
        assert abs(lhs - rhs) <= 1e-11 * float(np.abs(jv[k] * ut).sum()), (k, lhs, rhs)
