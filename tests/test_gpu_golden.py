"""The CUDA path against the golden fixtures made from the reference's own
routines (tests/golden/make_golden.py): boundary fills, residual, tangent,
adjoint, spanwise operators, norms and the colored-Jacobian indexing."""
import numpy as np
import pytest

from tests import golden_io as G
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _args(c):
    g, ph = c["grid"], c["phys"]
    return (g["x0"], g["y0"], g["nx"], g["ny"], g["xc"], g["yc"], g["vol"], g["volf"], g["gh"], ph["cp"], ph["cv"],
            ph["prandtl"], ph["gam"], ph["rgaz"], ph["cs"], ph["muref"], ph["tref"], ph["s_suth"], ph["k2"], ph["k4"])


@pytest.mark.parametrize("name", G.CASES)
def test_boundary_fills(name):
    d = G.load(name)
    c = G.as_case(d)
    w = d["w_raw"].copy(order="F")
    H.lib_bcs(c, w)
    assert np.abs(w - d["w"]).max() / np.abs(d["w"]).max() < 1e-13


@pytest.mark.parametrize("name", G.CASES)
def test_residual(name):
    from broadcast_gb300.srcfv import f_sch
    d = G.load(name)
    c = G.as_case(d)
    res = np.zeros_like(c["w"])
    f_sch.flux_num_dnc5_2d(res, c["w"], *_args(c))
    assert H.rel_err(res, d["res"], H.flux_scale(c, c["w"])) < 1e-12


@pytest.mark.parametrize("name", G.CASES)
def test_nowall_residual_and_tangent(name):
    from broadcast_gb300.srcfv import f_lin, f_sch
    d = G.load(name)
    c = G.as_case(d)
    res = np.zeros_like(c["w"])
    f_sch.flux_num_dnc5_nowall_2d(res, c["w"], *_args(c))
    assert H.rel_err(res, d["res_nowall"], H.flux_scale(c, c["w"])) < 1e-12
    r, rd = np.zeros_like(c["w"]), np.zeros_like(c["w"])
    f_lin.flux_num_dnc5_nowall_2d_d(r, rd, c["w"], np.asfortranarray(d["wd"][0]), *_args(c))
    sc = np.abs(H.interior(d["resd_nowall"])).reshape(-1, 5).max(0)
    assert H.rel_err(rd, d["resd_nowall"], sc) < 1e-11


@pytest.mark.parametrize("name", G.SCHEME_CASES)
def test_scheme_orders(name):
    """flux_num_dnc{3,7,9}[_nowall]_2d and _2d_d through the drop-in modules."""
    from broadcast_gb300.srcfv import f_lin, f_sch
    d = G.load(name)
    c = G.as_case(d)
    order, gh = int(d["order"]), int(d["gh"])
    for sfx in ("", "_nowall"):
        res = np.zeros_like(c["w"])
        getattr(f_sch, "flux_num_dnc%d%s_2d" % (order, sfx))(res, c["w"], *_args(c))
        assert H.rel_err(res, d["res" + sfx], H.flux_scale(c, c["w"]), gh) < 1e-12
        r, rd = np.zeros_like(c["w"]), np.zeros_like(c["w"])
        getattr(f_lin, "flux_num_dnc%d%s_2d_d" % (order, sfx))(r, rd, c["w"], np.asfortranarray(d["wd"]), *_args(c))
        assert H.rel_err(r, d["res" + sfx], H.flux_scale(c, c["w"]), gh) < 1e-12
        sc = np.abs(H.interior(d["resd" + sfx], gh)).reshape(-1, 5).max(0)
        assert H.rel_err(rd, d["resd" + sfx], sc, gh) < 1e-11


@pytest.mark.parametrize("name", G.NOWALL_ADJ_CASES)
def test_nowall_adjoint(name):
    """flux_num_dnc5_nowall_2d_b through srcfv.f_adj: wb on every padded cell,
    the interior of residub zeroed."""
    from broadcast_gb300.srcfv import f_adj
    d = G.load(name)
    c = G.as_case(d)
    rb = d["rb"].copy(order="F")
    wb = np.full_like(c["w"], 7.0)
    f_adj.flux_num_dnc5_nowall_2d_b(None, rb, c["w"], wb, *_args(c))
    sc = np.abs(d["wb_nowall"]).reshape(-1, 5).max(0)
    assert (np.abs(wb - d["wb_nowall"]).reshape(-1, 5).max(0) / sc).max() < 1e-11
    assert np.abs(rb[3:-3, 3:-3]).max() == 0.0


@pytest.mark.parametrize("name", G.IMPLI_CASES)
def test_impli_matrix_free(name):
    """impli_matrix_free_2d through srcfv.f_lhs: the whole dwi array."""
    from broadcast_gb300.srcfv import f_lhs
    d = G.load(name)
    c = G.as_case(d)
    g, ph = c["grid"], c["phys"]
    for lm in np.atleast_1d(d["lmax"]):
        dwi = np.full_like(c["w"], 3.0)
        f_lhs.impli_matrix_free_2d(dwi, g["nx"], g["ny"], c["w"], d["dw"], g["vol"], g["volf"], d["dtcoef"], d["cfl"],
                                   ph["gam"], ph["rgaz"], ph["prandtl"], int(lm), g["gh"], ph["cv"], ph["cs"],
                                   ph["muref"], ph["tref"], ph["cs"])
        ref = d["dwi_%d" % lm]
        assert np.abs(dwi - ref).max() <= 1e-12 * np.abs(ref).max(), lm


@pytest.mark.parametrize("name", G.CASES)
def test_tangent(name):
    from broadcast_gb300.srcfv import f_lin
    d = G.load(name)
    c = G.as_case(d)
    for k in range(d["wd"].shape[0]):
        res, resd = np.zeros_like(c["w"]), np.zeros_like(c["w"])
        f_lin.flux_num_dnc5_2d_d(res, resd, c["w"], np.asfortranarray(d["wd"][k]), *_args(c))
        sc = np.abs(H.interior(d["resd"][k])).reshape(-1, 5).max(0)
        assert H.rel_err(resd, d["resd"][k], sc) < 1e-11


@pytest.mark.parametrize("name", G.CASES)
@pytest.mark.parametrize("op", ["dz", "dzz"])
def test_spanwise_operators(name, op):
    from broadcast_gb300.srcfv import f_dz
    d = G.load(name)
    c = G.as_case(d)
    out = np.full_like(c["w"], 7.0)  # ghosts must stay untouched
    fn = f_dz.coeffs_5p_dz if op == "dz" else f_dz.coeffs_5p_dz2
    fn(out, c["w"], np.asfortranarray(d["wd"][0]), *_args(c)[:18])
    sc = np.maximum(np.abs(H.interior(d[op])).reshape(-1, 5).max(0), 1e-300)
    assert (np.abs(H.interior(out) - H.interior(d[op])).reshape(-1, 5).max(0) / sc).max() < 1e-12
    ghost = np.ones(out.shape, bool)
    ghost[3:-3, 3:-3] = False
    assert np.all(out[ghost] == 7.0)


def _fill_adjoint_cases():
    out = []
    for name in G.CASES:
        kinds = ("inlet", "noref", "extrap", "wall") if name.startswith("bl") else ("noref", "wall")
        out += [(name, k) for k in kinds]
    return out


@pytest.mark.parametrize("name,kind", _fill_adjoint_cases())
def test_fill_adjoints(name, kind):
    from broadcast_gb300.srcfv import f_adj
    d = G.load(name)
    c = G.as_case(d)
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    w = d["bcb_%s_w" % kind].copy(order="F")
    w0 = w.copy(order="F")
    wb = d["bcb_%s_in" % kind].copy(order="F")
    if kind == "inlet":
        f_adj.bc_supandsubinlet_2d_b(w, wb, "Ilo", it["Ilo"], c["field"], g["nx"], g["ny"], ph["gam"], im, jm)
    elif kind == "noref":
        f_adj.bc_no_reflexion_2d_b(w, wb, c["wbd"], "Jhi", it["Jhi"], g["nx"], g["ny"], ph["gam"], gh, im, jm)
    elif kind == "extrap":
        f_adj.bc_extrapolate_o2_2d_b(w, wb, "Ihi", it["Ihi"], im, jm, gh)
    else:
        f_adj.bc_wall_viscous_adia_2d_b(w, wb, "Jlo", ph["gam"], it["Jlo"], gh, im, jm)
    ref = d["bcb_%s_out" % kind]
    assert np.abs(wb - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.array_equal(w, w0)


def test_join_adjoint():
    from broadcast_gb300.srcfv import f_adj
    d = G.load("cyl_14x8")
    c = G.as_case(d)
    g, it = c["grid"], c["interf"]
    gh = g["gh"]
    wrb = d["jnb_wrb_in"].copy(order="F")
    wdb = np.full_like(wrb, 5.0)  # overwritten: zeroed, then accumulated
    f_adj.jn_match_2d_b(c["w"], wrb, it["prr1"], gh, gh, gh, gh, g["im"], g["jm"], c["w"], wdb, it["prd2"], gh, gh,
                        gh, gh, g["im"], g["jm"], it["tr"])
    assert np.array_equal(wrb, d["jnb_wrb_out"]) and np.array_equal(wdb, d["jnb_wdb_out"])


@pytest.mark.parametrize("name", G.CASES)
def test_adjoint(name):
    from broadcast_gb300.srcfv import f_adj
    d = G.load(name)
    c = G.as_case(d)
    wb = np.zeros_like(c["w"])
    f_adj.flux_num_dnc5_2d_b(None, d["rb"].copy(order="F"), c["w"], wb, *_args(c))
    sc = np.abs(d["wb"]).reshape(-1, 5).max(0)
    assert (np.abs(wb - d["wb"]).reshape(-1, 5).max(0) / sc).max() < 1e-11


@pytest.mark.parametrize("name", G.CASES)
def test_norms(name):
    from broadcast_gb300.srcfv import f_norm
    d = G.load(name)
    im, jm = int(d["im"]), int(d["jm"])
    a, b = f_norm.compute_norml2(d["res"], im, jm, 3)
    assert np.allclose(a, d["norml2"], rtol=1e-13, atol=0) and np.allclose(b, d["nmoy"], rtol=1e-13, atol=0)
    _, ninf = f_norm.compute_norml2inf(d["res"], im, jm, 3)
    assert np.allclose(ninf, d["ninf"], rtol=1e-12, atol=0)
    m, i, j = f_norm.compute_maxnorm(d["res"], im, jm, 3)
    assert np.array_equal(m, d["maxnorm"]) and np.array_equal(i, d["imax"]) and np.array_equal(j, d["jmax"])


def test_colored_indexing():
    from broadcast_gb300.misc import f_misc
    d = G.load("indexing_16x11")
    im, jm, gh = int(d["im"]), int(d["jm"]), int(d["gh"])
    nb = im * jm * 49 * 25
    for name in ("computejacobianfromjv", "computejacobianfromjv_relaxed", "computejacobianfromjv_relaxed_withjn",
                 "computejacobianfromjv_withjn", "computejacobianfromdz"):
        jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
        fn = getattr(f_misc, name)
        for (m, l, k) in d["seeds"]:
            if "relaxed" in name:
                fn(jac, ia, ja, d["resd"], int(m), int(l), int(k), gh, d["coefdiag"])
            else:
                fn(jac, ia, ja, d["resd"], int(m), int(l), int(k), gh)
        assert np.array_equal(jac, d[name + "_jac"]), name
        assert np.array_equal(ia, d[name + "_ia"]) and np.array_equal(ja, d[name + "_ja"]), name
    jac, ia, ja = np.zeros(2 * nb), np.zeros(2 * nb, np.int32), np.zeros(2 * nb, np.int32)
    for n in (0, 1):
        for (m, l, k) in d["seeds"]:
            f_misc.computejacobianfromjv_relaxed_withjnandcheck(jac, ia, ja, d["resd"], int(m), int(l), int(k), gh,
                                                                d["coefdiag"], 2e-16, n)
    assert np.array_equal(jac, d["check_jac"]) and np.array_equal(ia, d["check_ia"]) and np.array_equal(ja, d["check_ja"])
    for q, (m, l, k) in enumerate(d["seeds"]):
        wd = np.zeros((im + 6, jm + 6, 5), order="F")
        f_misc.testvector(wd, int(m), int(l), int(k), gh)
        assert np.array_equal(wd, d["testvectors"][2 * q])
        wd[:] = 0
        f_misc.testvector_partial(wd, int(m), int(l), int(k), gh, im, jm, 2, im - 2, 0, jm - 1)
        assert np.array_equal(wd, d["testvectors"][2 * q + 1])
