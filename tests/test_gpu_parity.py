"""Parity of the CUDA path (libbroadcast_gb300.so through its f2py-style
modules and the device operator API) against the CPU oracle.

Tolerances: residual within 1e-12 of the face-flux
magnitude (max-norm per variable); tangent outputs within 1e-11 of the same
scale times the tangent magnitude; boundary fills within 1e-13 relative;
integer index work bit-exact.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu

RES_TOL = 1e-12
JVP_TOL = 1e-11


def _prepared(kind, im, jm, seed=None):
    kw = {} if seed is None else {"seed": seed}
    c = H.bl_case(im, jm, **kw) if kind == "bl" else H.cyl_case(im, jm, **kw)
    H.oracle_bcs(c, c["w"])
    return c


def _args(c):
    g, ph = c["grid"], c["phys"]
    return (g["x0"], g["y0"], g["nx"], g["ny"], g["xc"], g["yc"], g["vol"], g["volf"], g["gh"], ph["cp"], ph["cv"],
            ph["prandtl"], ph["gam"], ph["rgaz"], ph["cs"], ph["muref"], ph["tref"], ph["s_suth"], ph["k2"], ph["k4"])


@pytest.mark.parametrize("kind,im,jm", [("bl", 40, 30), ("cyl", 28, 20), ("bl", 13, 9), ("cyl", 21, 7)])
def test_residual_host_arrays(kind, im, jm):
    from broadcast_gb300.srcfv import f_sch
    c = _prepared(kind, im, jm)
    ref = O.residual(c["grid"], c["phys"], c["w"])
    res = np.full_like(c["w"], 7.0)
    f_sch.flux_num_dnc5_2d(res, c["w"], *_args(c))
    assert np.isfinite(H.interior(res)).all()
    err = H.rel_err(res, ref, H.flux_scale(c, c["w"]))
    assert err < RES_TOL, err
    # ghosts of the output are left untouched, as in the reference
    assert (res[:3] == 7.0).all() and (res[:, -3:] == 7.0).all()


@pytest.mark.parametrize("kind,im,jm", [("bl", 400, 150), ("cyl", 256, 256)])
def test_residual_full_size_device(kind, im, jm):
    import torch
    from broadcast_gb300.operator import Dnc5Operator, to_device, to_host
    c = _prepared(kind, im, jm)
    ref = O.residual(c["grid"], c["phys"], c["w"])
    op = Dnc5Operator(c["grid"], c["phys"])
    res = op.residual(to_device(c["w"]))
    torch.cuda.synchronize()
    err = H.rel_err(to_host(res), ref, H.flux_scale(c, c["w"]))
    assert err < RES_TOL, err


@pytest.mark.parametrize("kind,im,jm", [("bl", 40, 30), ("cyl", 28, 20)])
def test_jvp_single_direction_host_arrays(kind, im, jm):
    from broadcast_gb300.srcfv import f_lin
    c = _prepared(kind, im, jm)
    rng = np.random.default_rng(3)
    wd = np.asfortranarray(rng.standard_normal(c["w"].shape))
    r0, rd0 = O.jvp(c["grid"], c["phys"], c["w"], wd)
    res, resd = np.zeros_like(c["w"]), np.zeros_like(c["w"])
    f_lin.flux_num_dnc5_2d_d(res, resd, c["w"], wd, *_args(c))
    sc = H.flux_scale(c, c["w"])
    assert H.rel_err(res, r0, sc) < RES_TOL
    tsc = np.abs(H.interior(rd0)).reshape(-1, 5).max(0)
    assert H.rel_err(resd, rd0, tsc) < JVP_TOL


@pytest.mark.parametrize("kind,im,jm,nd", [("bl", 40, 30, 7), ("cyl", 28, 20, 5), ("cyl", 256, 256, 4)])
def test_jvp_batched_device(kind, im, jm, nd):
    import torch
    from broadcast_gb300.operator import Dnc5Operator, to_device, to_host
    c = _prepared(kind, im, jm)
    rng = np.random.default_rng(4)
    wds = np.stack([np.asfortranarray(rng.standard_normal(c["w"].shape)) for _ in range(nd)])
    r0, rd0 = O.jvp(c["grid"], c["phys"], c["w"], wds)
    op = Dnc5Operator(c["grid"], c["phys"])
    wd_dev = torch.stack([to_device(x) for x in wds])
    res, resd = op.jvp(to_device(c["w"]), wd_dev)
    torch.cuda.synchronize()
    sc = H.flux_scale(c, c["w"])
    assert H.rel_err(to_host(res), r0, sc) < RES_TOL
    for k in range(nd):
        tsc = np.abs(H.interior(rd0[k])).reshape(-1, 5).max(0)
        assert H.rel_err(to_host(resd[k]), rd0[k], tsc) < JVP_TOL, k


@pytest.mark.parametrize("kind", ["bl", "cyl"])
def test_boundary_fills_match_oracle(kind):
    c = H.bl_case(40, 30) if kind == "bl" else H.cyl_case(28, 20)
    w0 = c["w"].copy(order="F")
    # scramble the ghosts so that every ghost value must come from the fill
    rng = np.random.default_rng(5)
    g = w0.copy(order="F")
    g[:3] += rng.uniform(0.1, 0.2, g[:3].shape)
    g[-3:] += rng.uniform(0.1, 0.2, g[-3:].shape)
    g[:, :3] += rng.uniform(0.1, 0.2, g[:, :3].shape)
    g[:, -3:] += rng.uniform(0.1, 0.2, g[:, -3:].shape)
    a, b = g.copy(order="F"), g.copy(order="F")
    H.oracle_bcs(c, a)
    H.lib_bcs(c, b)
    # one scale for all variables: the state magnitude (momenta of a
    # near-zero component still carry rounding of O(|w|) terms)
    scale = np.abs(a).max()
    assert np.abs(a - b).max() / scale < 1e-13
    # tangent fills
    wd = np.asfortranarray(rng.standard_normal(g.shape))
    a, b, ad, bd = g.copy(order="F"), g.copy(order="F"), wd.copy(order="F"), wd.copy(order="F")
    H.oracle_bcs(c, a, ad)
    H.lib_bcs(c, b, bd)
    assert np.abs(a - b).max() / scale < 1e-13
    assert np.abs(ad - bd).max() / np.abs(ad).max() < 1e-12


def test_norms_match_oracle():
    from broadcast_gb300.srcfv import f_norm
    c = _prepared("bl", 40, 30)
    r = O.residual(c["grid"], c["phys"], c["w"])
    a, b = f_norm.compute_norml2(r, 40, 30, 3)
    ea, eb = O.norml2(r, 40, 30, 3)
    assert np.allclose(a, ea, rtol=1e-13, atol=0) and np.allclose(b, eb, rtol=1e-13, atol=0)
    a, b = f_norm.compute_norml2inf(r, 40, 30, 3)
    ea, eb = O.norml2inf(r, 40, 30, 3)
    assert np.allclose(a, ea, rtol=1e-13, atol=0) and np.allclose(b, eb, rtol=1e-12, atol=0)
    a, i, j = f_norm.compute_maxnorm(r, 40, 30, 3)
    ea, ei, ej = O.maxnorm(r, 40, 30, 3)
    assert np.array_equal(a, ea) and np.array_equal(i, ei) and np.array_equal(j, ej)


@pytest.mark.parametrize("mode", ["plain", "relaxed", "relaxed_withjn", "withjn", "dz"])
def test_colored_indexing_bit_exact(mode):
    from broadcast_gb300.misc import f_misc
    im, jm, gh = 16, 11, 3
    rng = np.random.default_rng(6)
    resd = np.asfortranarray(rng.standard_normal((im + 6, jm + 6, 5)))
    coef = np.asfortranarray(rng.standard_normal((im, jm)))
    nb = im * jm * 49 * 25
    codes = dict(plain=O.JAC_PLAIN, relaxed=O.JAC_RELAXED, relaxed_withjn=O.JAC_RELAXED_WITHJN, withjn=O.JAC_WITHJN,
                 dz=O.JAC_DZ)
    for (m, l, k) in [(0, 0, 0), (2, 5, 1), (4, 6, 6), (1, 3, 4)]:
        ja_, ia_, jac_ = np.zeros(nb, np.int32), np.zeros(nb, np.int32), np.zeros(nb)
        jb_, ib_, jbc_ = np.zeros(nb, np.int32), np.zeros(nb, np.int32), np.zeros(nb)
        O.computejacobian(codes[mode], jac_, ia_, ja_, resd, m, l, k, gh, im, jm, coef if "relaxed" in mode else None)
        if mode == "plain":
            f_misc.computejacobianfromjv(jbc_, ib_, jb_, resd, m, l, k, gh)
        elif mode == "relaxed":
            f_misc.computejacobianfromjv_relaxed(jbc_, ib_, jb_, resd, m, l, k, gh, coef)
        elif mode == "relaxed_withjn":
            f_misc.computejacobianfromjv_relaxed_withjn(jbc_, ib_, jb_, resd, m, l, k, gh, coef)
        elif mode == "withjn":
            f_misc.computejacobianfromjv_withjn(jbc_, ib_, jb_, resd, m, l, k, gh)
        else:
            f_misc.computejacobianfromdz(jbc_, ib_, jb_, resd, m, l, k, gh)
        assert np.array_equal(ia_, ib_) and np.array_equal(ja_, jb_) and np.array_equal(jac_, jbc_)


def test_testvector_bit_exact():
    from broadcast_gb300.misc import f_misc
    im, jm, gh = 23, 17, 3
    for (m, l, k) in [(0, 0, 0), (3, 6, 2), (4, 1, 6)]:
        wd = np.full((im + 6, jm + 6, 5), 9.0, order="F")
        f_misc.testvector(wd, m, l, k, gh)
        assert np.array_equal(wd, O.testvector(m, l, k, gh, im, jm))
        wd[:] = 9.0
        f_misc.testvector_partial(wd, m, l, k, gh, im, jm, 2, 15, 0, 16)
        assert np.array_equal(wd, O.testvector_partial(m, l, k, gh, im, jm, 2, 15, 0, 16))


@pytest.mark.parametrize("kind,im,jm", [("bl", 40, 30), ("cyl", 64, 48)])
def test_nowall_matches_oracle(kind, im, jm):
    """flux_num_dnc5_nowall_2d (+ tangent): centred rows everywhere."""
    from broadcast_gb300.srcfv import f_lin, f_sch
    c = H.bl_case(im, jm) if kind == "bl" else H.cyl_case(im, jm)
    H.oracle_bcs(c, c["w"])
    g, ph = c["grid"], c["phys"]
    args = (g["x0"], g["y0"], g["nx"], g["ny"], g["xc"], g["yc"], g["vol"], g["volf"], g["gh"]) + tuple(
        ph[k] for k in ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4"))
    res = np.zeros_like(c["w"])
    f_sch.flux_num_dnc5_nowall_2d(res, c["w"], *args)
    assert H.rel_err(res, O.residual(g, ph, c["w"], nowall=True), H.flux_scale(c, c["w"])) < 1e-12
    rng = np.random.default_rng(7)
    wd = np.asfortranarray(rng.standard_normal(c["w"].shape))
    r, rd = np.zeros_like(res), np.zeros_like(res)
    f_lin.flux_num_dnc5_nowall_2d_d(r, rd, c["w"], wd, *args)
    _, ref = O.jvp(g, ph, c["w"], wd, nowall=True)
    sc = np.abs(H.interior(ref)).reshape(-1, 5).max(0)
    assert H.rel_err(rd, ref, sc) < 1e-11


@pytest.mark.parametrize("order", [3, 7, 9])
@pytest.mark.parametrize("kind,im,jm", [("bl", 40, 30), ("cyl", 64, 48)])
def test_scheme_orders_match_oracle(order, kind, im, jm):
    """flux_num_dnc{3,7,9}[_nowall]_2d (+ tangent) with the driver's ghost width
    gh = (order+1)//2, host arrays, against the oracle."""
    from broadcast_gb300.srcfv import f_lin, f_sch
    gh = (order + 1) // 2
    c = H.bl_case(im, jm, gh=gh) if kind == "bl" else H.cyl_case(im, jm, gh=gh)
    H.oracle_bcs(c, c["w"])
    g, ph = c["grid"], c["phys"]
    rng = np.random.default_rng(order)
    wd = np.asfortranarray(rng.standard_normal(c["w"].shape))
    for nowall, sfx in ((False, ""), (True, "_nowall")):
        res = np.full_like(c["w"], 7.0)
        getattr(f_sch, "flux_num_dnc%d%s_2d" % (order, sfx))(res, c["w"], *_args(c))
        ref = O.residual(g, ph, c["w"], nowall=nowall, order=order)
        assert H.rel_err(res, ref, H.flux_scale(c, c["w"]), gh) < RES_TOL
        assert (res[:gh] == 7.0).all() and (res[:, -gh:] == 7.0).all()
        r, rd = np.zeros_like(res), np.zeros_like(res)
        getattr(f_lin, "flux_num_dnc%d%s_2d_d" % (order, sfx))(r, rd, c["w"], wd, *_args(c))
        _, refd = O.jvp(g, ph, c["w"], wd, nowall=nowall, order=order)
        sc = np.abs(H.interior(refd, gh)).reshape(-1, 5).max(0)
        assert H.rel_err(rd, refd, sc, gh) < JVP_TOL


@pytest.mark.parametrize("order", [3, 7, 9])
def test_scheme_orders_device_arrays(order):
    """The same entry points on torch CUDA tensors (Fortran strides), queued on
    the library stream."""
    import torch
    from broadcast_gb300.operator import to_device, to_host
    from broadcast_gb300.srcfv import f_lin, f_sch
    gh = (order + 1) // 2
    c = H.bl_case(48, 36, gh=gh)
    H.oracle_bcs(c, c["w"])
    g, ph = c["grid"], c["phys"]
    dev = lambda a: to_device(a).permute(*reversed(range(a.ndim)))
    w = dev(c["w"])
    wd_h = np.asfortranarray(np.random.default_rng(5).standard_normal(c["w"].shape))
    args = (None, None, dev(g["nx"]), dev(g["ny"]), None, None, dev(g["vol"]), dev(g["volf"]), gh) + _args(c)[9:]
    res, r, rd = (dev(np.zeros_like(c["w"])) for _ in range(3))
    getattr(f_sch, "flux_num_dnc%d_2d" % order)(res, w, *args)
    getattr(f_lin, "flux_num_dnc%d_2d_d" % order)(r, rd, w, dev(wd_h), *args)
    torch.cuda.synchronize()
    host = lambda t: to_host(t.permute(*reversed(range(t.ndim))))
    ref = O.residual(g, ph, c["w"], order=order)
    assert H.rel_err(host(res), ref, H.flux_scale(c, c["w"]), gh) < RES_TOL
    _, refd = O.jvp(g, ph, c["w"], wd_h, order=order)
    sc = np.abs(H.interior(refd, gh)).reshape(-1, 5).max(0)
    assert H.rel_err(host(rd), refd, sc, gh) < JVP_TOL


def test_scheme_orders_reject_bad_extents():
    """Too few ghost layers for the stencil, or too few rows for the wall
    formulas, are refused before any launch."""
    from broadcast_gb300._lib import BroadcastError
    from broadcast_gb300.srcfv import f_sch
    c = H.bl_case(40, 30)  # gh = 3 < 5 needed by DNC9
    res = np.zeros_like(c["w"])
    with pytest.raises(BroadcastError):
        f_sch.flux_num_dnc9_2d(res, c["w"], *_args(c))
    c = H.bl_case(40, 8, gh=5)  # DNC9's wall rows read 11 cell rows
    res = np.zeros_like(c["w"])
    with pytest.raises(BroadcastError):
        f_sch.flux_num_dnc9_2d(res, c["w"], *_args(c))


def _impli(c, dw, lmax, cfl=5.0, dtcoef=1.0, dwi=None):
    from broadcast_gb300.srcfv import f_lhs
    g, ph = c["grid"], c["phys"]
    dwi = np.full_like(c["w"], 3.0) if dwi is None else dwi
    f_lhs.impli_matrix_free_2d(dwi, g["nx"], g["ny"], c["w"], dw, g["vol"], g["volf"], dtcoef, cfl, ph["gam"],
                               ph["rgaz"], ph["prandtl"], lmax, g["gh"], ph["cv"], ph["cs"], ph["muref"], ph["tref"],
                               ph["cs"])
    return dwi


@pytest.mark.parametrize("kind,im,jm,lmax", [("bl", 400, 150, 10), ("cyl", 64, 48, 10), ("bl", 40, 30, 3),
                                             ("cyl", 9, 7, 4)])
def test_impli_matrix_free_matches_oracle(kind, im, jm, lmax):
    """The cluster wavefront sweeps against the oracle's sequential loops, on the
    residual as the 'impli' time marching passes it (BROADCAST_npz.py:941)."""
    c = _prepared(kind, im, jm)
    g, ph = c["grid"], c["phys"]
    dw = O.residual(g, ph, c["w"])
    ref = O.impli_matrix_free(g, ph, c["w"], dw, 1.0, 5.0, lmax)
    dwi = _impli(c, dw, lmax)
    assert np.abs(dwi - ref).max() <= 1e-12 * np.abs(ref).max()
    gh = g["gh"]
    assert (dwi[:gh] == 0).all() and (dwi[-gh:] == 0).all() and (dwi[:, :gh] == 0).all() and (dwi[:, -gh:] == 0).all()


def test_impli_matrix_free_edge_cases():
    """lmax = 0 leaves dwi all zero; em != 5 is refused."""
    from broadcast_gb300._lib import BroadcastError
    from broadcast_gb300.srcfv import f_lhs
    c = _prepared("bl", 24, 16)
    g, ph = c["grid"], c["phys"]
    dw = O.residual(g, ph, c["w"])
    assert (_impli(c, dw, 0) == 0).all()
    dwi = np.zeros_like(c["w"])
    with pytest.raises(BroadcastError):
        f_lhs.impli_matrix_free_2d(dwi, g["nx"], g["ny"], c["w"], dw, g["vol"], g["volf"], 1.0, 5.0, ph["gam"],
                                   ph["rgaz"], ph["prandtl"], 2, g["gh"], ph["cv"], ph["cs"], ph["muref"], ph["tref"],
                                   ph["cs"], 24, 16, 4)


@pytest.mark.parametrize("gh", [2, 4, 5])
@pytest.mark.parametrize("kind", ["bl", "cyl"])
def test_boundary_fills_any_ghost_width(kind, gh):
    """The DNC3/7/9 drivers fill gh = 2, 4, 5 ghost layers with the same BC
    routines: the library's sequences (primal and tangent) against the oracle's."""
    c = H.bl_case(30, 20, gh=gh) if kind == "bl" else H.cyl_case(30, 20, gh=gh)
    w_ref, w_lib = c["w"].copy(order="F"), c["w"].copy(order="F")
    H.oracle_bcs(c, w_ref)
    H.lib_bcs(c, w_lib)
    assert np.abs(w_lib - w_ref).max() <= 1e-13 * np.abs(w_ref).max()
    rng = np.random.default_rng(gh)
    wd = np.asfortranarray(rng.standard_normal(c["w"].shape))
    wd_ref, wd_lib = wd.copy(order="F"), wd.copy(order="F")
    w2_ref, w2_lib = c["w"].copy(order="F"), c["w"].copy(order="F")
    H.oracle_bcs(c, w2_ref, wd_ref)
    H.lib_bcs(c, w2_lib, wd_lib)
    assert np.abs(wd_lib - wd_ref).max() <= 1e-12 * np.abs(wd_ref).max()
