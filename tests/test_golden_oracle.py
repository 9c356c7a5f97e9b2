"""The CPU oracle against the golden fixtures produced by the reference's own
routines (the parity pin of the oracle; runs everywhere, no GPU)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_io as G
from tests import helpers as H

# The oracle keeps the reference's evaluation order: on the machine that
# made the fixtures the residual is bit-identical; libm (tanh, pow) may differ
# by an ulp between platforms, hence the small tolerances.
TOL_RES = 1e-13
TOL_DERIV = 1e-12


@pytest.mark.parametrize("name", G.CASES)
def test_geometry_and_state(name):
    d = G.load(name)
    c = H.bl_case(d["im"], d["jm"], seed={"bl_14x10": 0, "bl_23x17": 3}[name]) if d["kind"] == "bl" else \
        H.cyl_case(d["im"], d["jm"], seed=1)
    for k in ("x0", "y0", "nx", "ny", "xc", "yc", "vol", "volf"):
        a, b = c["grid"][k], d[k]
        assert np.allclose(a, b, rtol=1e-14, atol=1e-14 * np.abs(b).max()), k
    assert np.allclose(c["w"], d["w_raw"], rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("name", G.CASES)
def test_boundary_fills(name):
    d = G.load(name)
    c = G.as_case(d)
    w = d["w_raw"].copy(order="F")
    H.oracle_bcs(c, w)
    assert np.abs(w - d["w"]).max() / np.abs(d["w"]).max() < 1e-14


@pytest.mark.parametrize("name", G.CASES)
def test_residual(name):
    d = G.load(name)
    c = G.as_case(d)
    r = O.residual(c["grid"], c["phys"], c["w"])
    assert H.rel_err(r, d["res"], H.flux_scale(c, c["w"])) < TOL_RES


@pytest.mark.parametrize("name", G.CASES)
def test_nowall_residual_and_tangent(name):
    """flux_num_dnc5_nowall_2d and its Tapenade tangent."""
    d = G.load(name)
    c = G.as_case(d)
    r = O.residual(c["grid"], c["phys"], c["w"], nowall=True)
    assert H.rel_err(r, d["res_nowall"], H.flux_scale(c, c["w"])) < TOL_RES
    _, rd = O.jvp(c["grid"], c["phys"], c["w"], d["wd"][0], nowall=True)
    sc = np.abs(H.interior(d["resd_nowall"])).reshape(-1, 5).max(0)
    assert H.rel_err(rd, d["resd_nowall"], sc) < TOL_DERIV


@pytest.mark.parametrize("name", G.SCHEME_CASES)
def test_scheme_orders(name):
    """flux_num_dnc{3,7,9}_2d, their tangents and the _nowall pairs."""
    d = G.load(name)
    c = G.as_case(d)
    order, gh = int(d["order"]), int(d["gh"])
    for nowall, sfx in ((False, ""), (True, "_nowall")):
        r = O.residual(c["grid"], c["phys"], c["w"], nowall=nowall, order=order)
        assert H.rel_err(r, d["res" + sfx], H.flux_scale(c, c["w"]), gh) < TOL_RES
        _, rd = O.jvp(c["grid"], c["phys"], c["w"], d["wd"], nowall=nowall, order=order)
        sc = np.abs(H.interior(d["resd" + sfx], gh)).reshape(-1, 5).max(0)
        assert H.rel_err(rd, d["resd" + sfx], sc, gh) < TOL_DERIV


@pytest.mark.parametrize("name", G.NOWALL_ADJ_CASES)
def test_nowall_adjoint(name):
    d = G.load(name)
    c = G.as_case(d)
    wb = O.vjp(c["grid"], c["phys"], c["w"], d["rb"], nowall=True)
    sc = np.abs(d["wb_nowall"]).reshape(-1, 5).max(0)
    assert (np.abs(wb - d["wb_nowall"]).reshape(-1, 5).max(0) / sc).max() < TOL_DERIV


@pytest.mark.parametrize("name", G.IMPLI_CASES)
def test_impli_matrix_free(name):
    """impli_matrix_free_2d: the whole dwi array (interior increment, zero ghosts)."""
    d = G.load(name)
    c = G.as_case(d)
    for lm in np.atleast_1d(d["lmax"]):
        dwi = O.impli_matrix_free(c["grid"], c["phys"], c["w"], d["dw"], d["dtcoef"], d["cfl"], int(lm))
        ref = d["dwi_%d" % lm]
        assert np.abs(dwi - ref).max() <= TOL_RES * np.abs(ref).max(), lm


@pytest.mark.parametrize("name", G.CASES)
def test_tangent(name):
    d = G.load(name)
    c = G.as_case(d)
    _, rd = O.jvp(c["grid"], c["phys"], c["w"], d["wd"])
    for k in range(d["wd"].shape[0]):
        sc = np.abs(H.interior(d["resd"][k])).reshape(-1, 5).max(0)
        assert H.rel_err(rd[k], d["resd"][k], sc) < TOL_DERIV


@pytest.mark.parametrize("name", G.CASES)
def test_adjoint(name):
    d = G.load(name)
    c = G.as_case(d)
    wb = O.vjp(c["grid"], c["phys"], c["w"], d["rb"])
    sc = np.abs(d["wb"]).reshape(-1, 5).max(0)
    assert (np.abs(wb - d["wb"]).reshape(-1, 5).max(0) / sc).max() < TOL_DERIV


@pytest.mark.parametrize("name", G.CASES)
@pytest.mark.parametrize("op", ["dz", "dzz"])
def test_spanwise_operators(name, op):
    """coeffs_5p_dz / coeffs_5p_dz2 on the first tangent direction; ghosts untouched."""
    d = G.load(name)
    c = G.as_case(d)
    fn = O.dz if op == "dz" else O.dzz
    got = fn(c["grid"], c["phys"], c["w"], d["wd"][0])
    sc = np.maximum(np.abs(H.interior(d[op])).reshape(-1, 5).max(0), 1e-300)
    assert (np.abs(got - d[op]).reshape(-1, 5).max(0) / sc).max() < TOL_DERIV
    assert not np.any(got[:3]) and not np.any(got[-3:]) and not np.any(got[:, :3]) and not np.any(got[:, -3:])


def _fill_adjoint_cases():
    out = []
    for name in G.CASES:
        kinds = ("inlet", "noref", "extrap", "wall") if name.startswith("bl") else ("noref", "wall")
        out += [(name, k) for k in kinds]
    return out


LOCS = {"inlet": "Ilo", "noref": "Jhi", "extrap": "Ihi", "wall": "Jlo"}


@pytest.mark.parametrize("name,kind", _fill_adjoint_cases())
def test_fill_adjoints(name, kind):
    """Transposes of the ghost fills against adjoint/bc_*_b.f90."""
    d = G.load(name)
    c = G.as_case(d)
    g, ph = c["grid"], c["phys"]
    loc = LOCS[kind]
    wb = d["bcb_%s_in" % kind].copy(order="F")
    aux = {"inlet": c.get("field"), "noref": c["wbd"]}.get(kind)
    O.bc_adjoint(kind, d["bcb_%s_w" % kind], wb, loc, c["interf"][loc], g["gh"], g["im"], g["jm"], gam=ph["gam"],
                 aux=aux, nx=g["nx"], ny=g["ny"])
    ref = d["bcb_%s_out" % kind]
    assert np.abs(wb - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("name", G.CASES)
def test_norms(name):
    d = G.load(name)
    im, jm = int(d["im"]), int(d["jm"])
    a, b = O.norml2(d["res"], im, jm, 3)
    assert np.array_equal(a, d["norml2"]) and np.array_equal(b, d["nmoy"])
    _, ninf = O.norml2inf(d["res"], im, jm, 3)
    assert np.allclose(ninf, d["ninf"], rtol=1e-14, atol=0)
    m, i, j = O.maxnorm(d["res"], im, jm, 3)
    assert np.array_equal(m, d["maxnorm"]) and np.array_equal(i, d["imax"]) and np.array_equal(j, d["jmax"])


def test_colored_indexing():
    d = G.load("indexing_16x11")
    im, jm, gh = int(d["im"]), int(d["jm"]), int(d["gh"])
    nb = im * jm * 49 * 25
    modes = {"computejacobianfromjv": O.JAC_PLAIN, "computejacobianfromjv_relaxed": O.JAC_RELAXED,
             "computejacobianfromjv_relaxed_withjn": O.JAC_RELAXED_WITHJN,
             "computejacobianfromjv_withjn": O.JAC_WITHJN, "computejacobianfromdz": O.JAC_DZ}
    for name, mode in modes.items():
        jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
        for (m, l, k) in d["seeds"]:
            O.computejacobian(mode, jac, ia, ja, d["resd"], int(m), int(l), int(k), gh, im, jm,
                              d["coefdiag"] if "relaxed" in name else None)
        assert np.array_equal(jac, d[name + "_jac"]), name
        assert np.array_equal(ia, d[name + "_ia"]) and np.array_equal(ja, d[name + "_ja"]), name
    jac, ia, ja = np.zeros(2 * nb), np.zeros(2 * nb, np.int32), np.zeros(2 * nb, np.int32)
    for n in (0, 1):
        for (m, l, k) in d["seeds"]:
            O.computejacobian_withjnandcheck(jac, ia, ja, d["resd"], int(m), int(l), int(k), gh, im, jm, d["coefdiag"],
                                             2e-16, n)
    assert np.array_equal(jac, d["check_jac"]) and np.array_equal(ia, d["check_ia"]) and np.array_equal(ja, d["check_ja"])
    for q, (m, l, k) in enumerate(d["seeds"]):
        assert np.array_equal(O.testvector(int(m), int(l), int(k), gh, im, jm), d["testvectors"][2 * q])
        assert np.array_equal(O.testvector_partial(int(m), int(l), int(k), gh, im, jm, 2, im - 2, 0, jm - 1),
                              d["testvectors"][2 * q + 1])
