"""Parity of the CUDA adjoint (VJP) with the oracle, the dot-product identity
<J v, u> = <v, J^T u>, and the reference's in-place semantics."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu
TOL = 1e-11


def _args(c):
    g, ph = c["grid"], c["phys"]
    return (g["x0"], g["y0"], g["nx"], g["ny"], g["xc"], g["yc"], g["vol"], g["volf"], g["gh"], ph["cp"], ph["cv"],
            ph["prandtl"], ph["gam"], ph["rgaz"], ph["cs"], ph["muref"], ph["tref"], ph["s_suth"], ph["k2"], ph["k4"])


@pytest.mark.parametrize("kind,im,jm", [("bl", 40, 30), ("cyl", 28, 20), ("bl", 13, 9), ("cyl", 64, 48)])
def test_vjp_matches_oracle(kind, im, jm):
    from broadcast_gb300.srcfv import f_adj
    c = H.bl_case(im, jm) if kind == "bl" else H.cyl_case(im, jm)
    H.oracle_bcs(c, c["w"])
    rng = np.random.default_rng(11)
    rb = np.zeros_like(c["w"])
    rb[3:-3, 3:-3] = rng.standard_normal((im, jm, 5))
    ref = O.vjp(c["grid"], c["phys"], c["w"], rb)
    rb_gpu = rb.copy(order="F")
    wb = np.full_like(c["w"], 5.0)
    f_adj.flux_num_dnc5_2d_b(None, rb_gpu, c["w"], wb, *_args(c))
    assert np.all(rb_gpu[3:-3, 3:-3] == 0.0)  # consumed, as in the reference
    sc = np.abs(ref).reshape(-1, 5).max(0)
    err = (np.abs(wb - ref).reshape(-1, 5).max(0) / sc).max()
    assert err < TOL, err


def test_dot_product_identity():
    from broadcast_gb300.srcfv import f_adj, f_lin
    c = H.cyl_case(40, 24)
    H.oracle_bcs(c, c["w"])
    rng = np.random.default_rng(12)
    v = np.asfortranarray(rng.standard_normal(c["w"].shape))
    u = np.zeros_like(c["w"])
    u[3:-3, 3:-3] = rng.standard_normal((40, 24, 5))
    res, jv = np.zeros_like(v), np.zeros_like(v)
    f_lin.flux_num_dnc5_2d_d(res, jv, c["w"], v, *_args(c))
    wb = np.zeros_like(v)
    f_adj.flux_num_dnc5_2d_b(None, u.copy(order="F"), c["w"], wb, *_args(c))
    a, b = np.sum(H.interior(jv) * H.interior(u)), np.sum(v * wb)
    assert abs(a - b) <= 1e-12 * max(abs(a), abs(b)), (a, b)


def test_boundary_chain_adjoint_dot_product():
    """Full boundary-layer chain (inlet, no-reflexion, extrapolation, wall):
    <T x, y> = <x, T^T y> with the tangent fills forward and the fill
    adjoints in reverse order, on the GPU, against the oracle's adjoints."""
    from broadcast_gb300.srcfv import f_adj, f_lin
    c = H.bl_case(64, 40)
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    rng = np.random.default_rng(21)
    x = np.asfortranarray(rng.standard_normal(c["w"].shape))
    y = np.asfortranarray(rng.standard_normal(c["w"].shape))
    # states before each fill
    states = []
    w = c["w"].copy(order="F")
    steps = [("inlet", "Ilo"), ("noref", "Jhi"), ("extrap", "Ihi"), ("wall", "Jlo")]
    tx = x.copy(order="F")
    for kind, loc in steps:
        states.append(w.copy(order="F"))
        if kind == "inlet":
            f_lin.bc_supandsubinlet_2d_d(w, tx, loc, it[loc], c["field"], g["nx"], g["ny"], ph["gam"], im, jm)
        elif kind == "noref":
            f_lin.bc_no_reflexion_2d_d(w, tx, c["wbd"], loc, it[loc], g["nx"], g["ny"], ph["gam"], gh, im, jm)
        elif kind == "extrap":
            f_lin.bc_extrapolate_o2_2d_d(w, tx, loc, it[loc], im, jm, gh)
        else:
            f_lin.bc_wall_viscous_adia_2d_d(w, tx, loc, ph["gam"], it[loc], gh, im, jm)
    ty = y.copy(order="F")
    oy = y.copy(order="F")
    for (kind, loc), ws in zip(reversed(steps), reversed(states)):
        wcopy = ws.copy(order="F")
        aux = {"inlet": c["field"], "noref": c["wbd"]}.get(kind)
        O.bc_adjoint(kind, ws, oy, loc, it[loc], gh, im, jm, gam=ph["gam"], aux=aux, nx=g["nx"], ny=g["ny"])
        if kind == "inlet":
            f_adj.bc_supandsubinlet_2d_b(wcopy, ty, loc, it[loc], c["field"], g["nx"], g["ny"], ph["gam"], im, jm)
        elif kind == "noref":
            f_adj.bc_no_reflexion_2d_b(wcopy, ty, c["wbd"], loc, it[loc], g["nx"], g["ny"], ph["gam"], gh, im, jm)
        elif kind == "extrap":
            f_adj.bc_extrapolate_o2_2d_b(wcopy, ty, loc, it[loc], im, jm, gh)
        else:
            f_adj.bc_wall_viscous_adia_2d_b(wcopy, ty, loc, ph["gam"], it[loc], gh, im, jm)
        assert np.array_equal(wcopy, ws)
    assert np.abs(ty - oy).max() <= 1e-12 * np.abs(oy).max()
    lhs, rhs = float(np.vdot(tx, y)), float(np.vdot(x, ty))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), np.abs(tx).max() * np.abs(y).sum())


@pytest.mark.parametrize("kind,im,jm", [("bl", 40, 30), ("cyl", 28, 20)])
def test_nowall_vjp_matches_oracle_and_tangent(kind, im, jm):
    """flux_num_dnc5_nowall_2d_b: against the oracle, and <J v, u> = <v, J^T u>
    with the GPU tangent of the same scheme (flux_num_dnc5_nowall_2d_d)."""
    from broadcast_gb300.srcfv import f_adj, f_lin
    c = H.bl_case(im, jm) if kind == "bl" else H.cyl_case(im, jm)
    H.oracle_bcs(c, c["w"])
    rng = np.random.default_rng(12)
    u = np.zeros_like(c["w"])
    u[3:-3, 3:-3] = rng.standard_normal((im, jm, 5))
    ref = O.vjp(c["grid"], c["phys"], c["w"], u, nowall=True)
    ub = u.copy(order="F")
    wb = np.full_like(c["w"], 5.0)
    f_adj.flux_num_dnc5_nowall_2d_b(None, ub, c["w"], wb, *_args(c))
    assert np.all(ub[3:-3, 3:-3] == 0.0)
    sc = np.abs(ref).reshape(-1, 5).max(0)
    assert (np.abs(wb - ref).reshape(-1, 5).max(0) / sc).max() < TOL
    v = np.asfortranarray(rng.standard_normal(c["w"].shape))
    r, jv = np.zeros_like(c["w"]), np.zeros_like(c["w"])
    f_lin.flux_num_dnc5_nowall_2d_d(r, jv, c["w"], v, *_args(c))
    lhs = float(np.sum(H.interior(jv) * H.interior(u)))
    rhs = float(np.sum(v * wb))
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), abs(rhs))


@pytest.mark.parametrize("nd", [1, 3])
def test_batched_vjp_equals_single_calls(nd):
    """bcg_flux_num_dnc5_2d_bn: nd cotangents in one call (host arrays), bit
    for bit the results of nd calls of flux_num_dnc5_2d_b, every residub
    interior consumed."""
    from broadcast_gb300 import _lib
    from broadcast_gb300.srcfv import f_adj
    c = H.cyl_case(40, 24)
    H.oracle_bcs(c, c["w"])
    rng = np.random.default_rng(31)
    rbs = np.zeros(c["w"].shape + (nd,), order="F")
    rbs[3:-3, 3:-3] = rng.standard_normal((40, 24, 5, nd))
    rb_in = rbs.copy(order="F")
    wbs = np.full_like(rbs, 7.0)
    _lib.call("bcg_flux_num_dnc5_2d_bn", None, rbs, c["w"], wbs, nd, *_args(c), 40, 24)
    assert np.all(rbs[3:-3, 3:-3] == 0.0)
    for k in range(nd):
        wb = np.zeros_like(c["w"])
        f_adj.flux_num_dnc5_2d_b(None, rb_in[..., k].copy(order="F"), c["w"], wb, *_args(c))
        assert np.array_equal(wbs[..., k], wb), k


def test_batched_vjp_device_arrays():
    """The operator's batched VJP (device arrays, K cotangents in one call)
    equals K single-cotangent calls bit for bit, and matches the oracle."""
    import torch
    from broadcast_gb300.operator import Dnc5Operator, to_device, to_host
    c = H.cyl_case(32, 20)
    H.oracle_bcs(c, c["w"])
    op = Dnc5Operator(c["grid"], c["phys"])
    w = to_device(c["w"])
    rng = np.random.default_rng(32)
    k = 5
    rbs = torch.zeros((k,) + tuple(op.state_shape), dtype=torch.float64, device="cuda")
    rbs[:, :, 3:-3, 3:-3] = torch.from_numpy(rng.standard_normal((k, 5, 20, 32))).cuda()
    wbs = op.vjp(w, rbs)
    torch.cuda.synchronize()
    for i in range(k):
        wb1 = op.vjp(w, rbs[i])
        assert torch.equal(wbs[i], wb1), i
    rb0 = to_host(rbs[2], c["w"].shape)
    ref = O.vjp(c["grid"], c["phys"], c["w"], rb0)
    got = to_host(wbs[2], c["w"].shape)
    sc = np.abs(ref).reshape(-1, 5).max(0)
    assert (np.abs(got - ref).reshape(-1, 5).max(0) / sc).max() < TOL
