"""The f2py-compatible modules against the C ABI, without a GPU.

Every routine of broadcast_gb300.srcfv.f_*, misc.f_misc and f_init is called
in the reference drivers' form (BROADCAST_npz.py:1018-1031,1072-1127,1221-1249,
cylinder.py:481-527,602-612,889-981, handleBC.py:142-181), with trailing
dimensions given and omitted, while the library call is recorded instead of
run.  Each recorded call must name a declared entry point with its
signature's arity, and carry the caller's arrays (the same objects: in-place
arguments are not copied), interface ranges, location strings and scalars in
the header's parameter order (include/broadcast_gb300.h), with the dimensions
f2py would infer.
"""
import numpy as np
import pytest

from broadcast_gb300 import _lib, f_init
from broadcast_gb300.misc import f_misc
from broadcast_gb300.srcfv import f_adj, f_bnd, f_dz, f_geom, f_lhs, f_lin, f_norm, f_sch
from tests import helpers as H


class IF:
    """An interface range given as the drivers' (2, 2) array: passed as
    column-major int32 {imin, imax, jmin, jmax}."""

    def __init__(self, a):
        self.v = np.asarray(a).reshape(2, 2).T.ravel().astype(np.int32)

    def ok(self, x):
        return isinstance(x, np.ndarray) and x.dtype == np.int32 and np.array_equal(x, self.v)


class LOC:
    def __init__(self, s):
        self.s = s

    def ok(self, x):
        b = x.encode() if isinstance(x, str) else bytes(x)
        return b[:3] == self.s.encode()


class I32:
    """An int32 array with these values (the join's transform)."""

    def __init__(self, a):
        self.v = np.asarray(a, dtype=np.int32).ravel()

    def ok(self, x):
        return isinstance(x, np.ndarray) and x.dtype == np.int32 and np.array_equal(x.ravel(), self.v)


def _match(got, want):
    if isinstance(want, (IF, LOC, I32)):
        return want.ok(got)
    if want is None:
        return got is None
    if isinstance(want, np.ndarray):
        return got is want
    return type(got) in (int, float, np.int32, np.int64, np.float64) and got == want


@pytest.fixture()
def recorder(monkeypatch):
    calls = []
    monkeypatch.setattr(_lib, "call", lambda name, *args: calls.append((name, args)) or 0)
    return calls


def _phys(ph):
    return [ph[k] for k in ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref")]


def _bl():
    c = H.bl_case(20, 16, seed=1)
    g = c["grid"]
    z = lambda: np.zeros_like(c["w"], order="F")
    return c, g, c["phys"], z


def _check(calls, expected):
    assert len(calls) == len(expected), [n for n, _ in calls]
    for (name, args), (sym, want) in zip(calls, expected):
        assert name == sym, (name, sym)
        assert name in _lib.SIGNATURES
        assert len(args) == len(_lib.SIGNATURES[name]) == len(want), (name, len(args), len(want))
        for q, (a, b) in enumerate(zip(args, want)):
            assert _match(a, b), (name, q, a if not isinstance(a, np.ndarray) else a.shape)


def test_residual_tangent_adjoint_and_spanwise(recorder):
    c, g, ph, z = _bl()
    gh, im, jm = g["gh"], g["im"], g["jm"]
    x0, y0, nx, ny, xc, yc, vol, volf = (g[k] for k in ("x0", "y0", "nx", "ny", "xc", "yc", "vol", "volf"))
    w, wd, res, resd, wb, rb, dz = c["w"], z(), z(), z(), z(), z(), z()
    cp, cv, pr, gam, rgaz, cs, muref, tref = _phys(ph)
    k2, k4 = ph["k2"], ph["k4"]
    common = (x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, pr, gam, rgaz, cs, muref, tref, cs, k2, k4)
    ptrs = [None, None, nx, ny, None, None, vol, volf, gh, cp, cv, pr, gam, rgaz, cs, muref, tref, cs, k2, k4, im, jm]
    f_sch.flux_num_dnc5_2d(res, w, *common, im, jm)                        # BROADCAST_npz.py:1031
    f_sch.flux_num_dnc5_2d(res, w, *common)                                # trailing dimensions inferred
    f_sch.flux_num_dnc5_nowall_2d(res, w, *common, im, jm)
    f_sch.flux_num_dnc9_2d(res, w, *common, im, jm)
    f_lin.flux_num_dnc5_2d_d(res, resd, w, wd, *common, im, jm)            # BROADCAST_npz.py:1085
    f_lin.flux_num_dnc7_nowall_2d_d(res, resd, w, wd, *common)
    f_adj.flux_num_dnc5_2d_b(res, rb, w, wb, *common, im, jm)
    f_adj.flux_num_dnc5_nowall_2d_b(res, rb, w, wb, *common)
    f_dz.coeffs_5p_dz(dz, w, wd, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, pr, gam, rgaz, cs, muref, tref, cs,
                      im, jm)                                               # BROADCAST_npz.py:1240
    f_dz.coeffs_5p_dz2(dz, w, wd, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, pr, gam, rgaz, cs, muref, tref, cs)
    span = [None, None, nx, ny, None, None, vol, None, gh, cp, cv, pr, gam, rgaz, cs, muref, tref, cs, im, jm]
    _check(recorder, [
        ("bcg_flux_num_dnc5_2d", [res, w] + ptrs),
        ("bcg_flux_num_dnc5_2d", [res, w] + ptrs),
        ("bcg_flux_num_dnc5_nowall_2d", [res, w] + ptrs),
        ("bcg_flux_num_dnc9_2d", [res, w] + ptrs),
        ("bcg_flux_num_dnc5_2d_d", [res, resd, w, wd] + ptrs),
        ("bcg_flux_num_dnc7_nowall_2d_d", [res, resd, w, wd] + ptrs),
        ("bcg_flux_num_dnc5_2d_b", [None, rb, w, wb] + ptrs),          # residu is not used by the adjoint
        ("bcg_flux_num_dnc5_nowall_2d_b", [None, rb, w, wb] + ptrs),
        ("bcg_coeffs_5p_dz", [dz, w, wd] + span),
        ("bcg_coeffs_5p_dz2", [dz, w, wd] + span),
    ])


def test_boundary_fills_tangents_and_adjoints(recorder):
    c, g, ph, z = _bl()
    gh, im, jm = g["gh"], g["im"], g["jm"]
    nx, ny, gam = g["nx"], g["ny"], ph["gam"]
    w, wd, wb, field, wbd, it = c["w"], z(), z(), c["field"], c["wbd"], c["interf"]
    lf, lb = field.shape[0], wbd.shape[0]
    # BROADCAST_npz.py:1018-1021 and the tangent chain :1079-1082
    f_bnd.bc_supandsubinlet_2d(w, "Ilo", it["Ilo"], field, nx, ny, gam, im, jm)
    f_bnd.bc_no_reflexion_2d(w, wbd, "Jhi", it["Jhi"], nx, ny, gam, gh, im, jm)
    f_bnd.bc_extrapolate_o2_2d(w, "Ihi", it["Ihi"], im, jm, gh)
    f_bnd.bc_wall_viscous_adia_2d(w, "Jlo", gam, it["Jlo"], gh, im, jm)
    f_lin.bc_supandsubinlet_2d_d(w, wd, "Ilo", it["Ilo"], field, nx, ny, gam, im, jm)
    f_lin.bc_no_reflexion_2d_d(w, wd, wbd, "Jhi", it["Jhi"], nx, ny, gam, gh, im, jm)
    f_lin.bc_extrapolate_o2_2d_d(w, wd, "Ihi", it["Ihi"], im, jm, gh)
    f_lin.bc_wall_viscous_adia_2d_d(w, wd, "Jlo", gam, it["Jlo"], gh, im, jm)
    f_adj.bc_supandsubinlet_2d_b(w, wb, "Ilo", it["Ilo"], field, nx, ny, gam, im, jm)
    f_adj.bc_no_reflexion_2d_b(w, wb, wbd, "Jhi", it["Jhi"], nx, ny, gam, gh, im, jm)
    f_adj.bc_extrapolate_o2_2d_b(w, wb, "Ihi", it["Ihi"], im, jm, gh)
    f_adj.bc_wall_viscous_adia_2d_b(w, wb, "Jlo", gam, it["Jlo"], gh, im, jm)
    _check(recorder, [
        ("bcg_bc_supandsubinlet_2d", [w, LOC("Ilo"), IF(it["Ilo"]), field, nx, ny, gam, im, jm, lf, gh]),
        ("bcg_bc_no_reflexion_2d", [w, wbd, LOC("Jhi"), IF(it["Jhi"]), nx, ny, gam, gh, im, jm, lb]),
        ("bcg_bc_extrapolate_o2_2d", [w, LOC("Ihi"), IF(it["Ihi"]), im, jm, gh, 5]),
        ("bcg_bc_wall_viscous_adia_2d", [w, LOC("Jlo"), gam, IF(it["Jlo"]), gh, im, jm]),
        ("bcg_bc_supandsubinlet_2d_d", [w, wd, LOC("Ilo"), IF(it["Ilo"]), field, nx, ny, gam, im, jm, lf, gh]),
        ("bcg_bc_no_reflexion_2d_d", [w, wd, wbd, LOC("Jhi"), IF(it["Jhi"]), nx, ny, gam, gh, im, jm, lb]),
        ("bcg_bc_extrapolate_o2_2d_d", [w, wd, LOC("Ihi"), IF(it["Ihi"]), im, jm, gh, 5]),
        ("bcg_bc_wall_viscous_adia_2d_d", [w, wd, LOC("Jlo"), gam, IF(it["Jlo"]), gh, im, jm]),
        ("bcg_bc_supandsubinlet_2d_b", [w, wb, LOC("Ilo"), IF(it["Ilo"]), field, nx, ny, gam, im, jm, lf, gh]),
        ("bcg_bc_no_reflexion_2d_b", [w, wb, wbd, LOC("Jhi"), IF(it["Jhi"]), nx, ny, gam, gh, im, jm, lb]),
        ("bcg_bc_extrapolate_o2_2d_b", [w, wb, LOC("Ihi"), IF(it["Ihi"]), im, jm, gh, 5]),
        ("bcg_bc_wall_viscous_adia_2d_b", [w, wb, LOC("Jlo"), gam, IF(it["Jlo"]), gh, im, jm]),
    ])


def test_periodic_joins(recorder):
    """cylinder.py:481-527 (metric joins) and the state joins of
    handleBC.applyBC (prr/prd ranges, tr = [1, 2])."""
    c = H.cyl_case(21, 14, seed=1)
    g, it = c["grid"], c["interf"]
    gh, im, jm = g["gh"], g["im"], g["jm"]
    w = c["w"]
    wd, wb, wdb = (np.zeros_like(w, order="F") for _ in range(3))
    vol, tr = g["vol"], it["tr"]
    f_bnd.jn_match_geom_2d(vol, it["prr1"], gh, gh, gh, gh, im, jm, vol, it["prd2"], gh, gh, gh, gh, im, jm, tr)
    f_bnd.jn_match_2d(w, it["prr1"], gh, gh, gh, gh, im, jm, w, it["prd2"], gh, gh, gh, gh, im, jm, tr)
    f_lin.jn_match_2d_d(w, wd, it["prr2"], gh, gh, gh, gh, im, jm, w, wd, it["prd1"], gh, gh, gh, gh, im, jm, tr)
    f_adj.jn_match_2d_b(w, wb, it["prr1"], gh, gh, gh, gh, im, jm, w, wdb, it["prd2"], gh, gh, gh, gh, im, jm, tr)
    g4 = [gh] * 4
    _check(recorder, [
        ("bcg_jn_match_geom_2d", [vol, IF(it["prr1"])] + g4 + [im, jm, vol, IF(it["prd2"])] + g4 + [im, jm, I32(tr)]),
        ("bcg_jn_match_2d", [w, IF(it["prr1"])] + g4 + [im, jm, w, IF(it["prd2"])] + g4 + [im, jm, I32(tr), 5]),
        ("bcg_jn_match_2d_d", [w, wd, IF(it["prr2"])] + g4 + [im, jm, w, wd, IF(it["prd1"])] + g4
         + [im, jm, I32(tr), 5]),
        ("bcg_jn_match_2d_b", [None, wb, IF(it["prr1"])] + g4 + [im, jm, None, wdb, IF(it["prd2"])] + g4
         + [im, jm, I32(tr), 5]),
    ])


def test_seeding_fills_norms_geometry_init_and_implicit_phase(recorder):
    c, g, ph, z = _bl()
    gh, im, jm = g["gh"], g["im"], g["jm"]
    nb = im * jm * 49 * 25
    jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
    jac2, ia2, ja2 = np.zeros(2 * nb), np.zeros(2 * nb, np.int32), np.zeros(2 * nb, np.int32)
    wd, resd, res, dwi = z(), z(), z(), z()
    cd = np.asfortranarray(np.ones((im, jm)))
    f_misc.testvector(wd, 2, 3, 4, gh, im, jm)                                   # BROADCAST_npz.py:1074
    f_misc.testvector(wd, 2, 3, 4, gh)
    f_misc.testvector_partial(wd, 1, 0, 6, gh, im, jm, 0, 6, 0, jm - 1)          # cylinder.py:905
    f_misc.computejacobianfromjv(jac, ia, ja, resd, 1, 2, 3, gh, im, jm)
    f_misc.computejacobianfromjv_relaxed(jac, ia, ja, resd, 1, 2, 3, gh, cd)    # BROADCAST_npz.py:1127
    f_misc.computejacobianfromjv_relaxed_withjn(jac, ia, ja, resd, 1, 2, 3, gh, cd, im, jm)
    f_misc.computejacobianfromjv_withjn(jac, ia, ja, resd, 1, 2, 3, gh)
    f_misc.computejacobianfromjv_relaxed_withjnandcheck(jac2, ia2, ja2, resd, 1, 2, 3, gh, cd, 2e-16, 1)
    f_misc.computejacobianfromdz(jac, ia, ja, resd, 4, 0, 6, gh, im, jm)        # BROADCAST_npz.py:1243
    n2, m2 = f_norm.compute_norml2(res, im, jm, gh)
    n3, m3 = f_norm.compute_norml2inf(res)
    n4, i4, j4 = f_norm.compute_maxnorm(res, im, jm, gh)
    geo = [g[k] for k in ("x0", "y0", "nx", "ny", "xc", "yc", "vol", "volf")]
    f_geom.computegeom_2d(*geo, im, jm, gh)                                      # cylinder.py:497
    f_init.initblfv(ph["muinf"], g["xc"], g["yc"], c["w"], c["field"], im, gh, jm)
    f_init.set_bndbl_2d(c["w"], c["field"], c["wbd"], im, jm, gh)
    f_lhs.impli_matrix_free_2d(dwi, g["nx"], g["ny"], c["w"], res, g["vol"], g["volf"], 1.0, 5.0, ph["gam"],
                               ph["rgaz"], ph["prandtl"], 10, gh, ph["cv"], ph["cs"], ph["muref"], ph["tref"],
                               ph["cs"], im, jm)
    _check(recorder, [
        ("bcg_testvector", [wd, 2, 3, 4, gh, im, jm]),
        ("bcg_testvector", [wd, 2, 3, 4, gh, im, jm]),
        ("bcg_testvector_partial", [wd, 1, 0, 6, gh, im, jm, 0, 6, 0, jm - 1]),
        ("bcg_computejacobianfromjv", [jac, ia, ja, resd, 1, 2, 3, gh, im, jm, nb]),
        ("bcg_computejacobianfromjv_relaxed", [jac, ia, ja, resd, 1, 2, 3, gh, im, jm, nb, cd]),
        ("bcg_computejacobianfromjv_relaxed_withjn", [jac, ia, ja, resd, 1, 2, 3, gh, im, jm, nb, cd]),
        ("bcg_computejacobianfromjv_withjn", [jac, ia, ja, resd, 1, 2, 3, gh, im, jm, nb]),
        ("bcg_computejacobianfromjv_relaxed_withjnandcheck",
         [jac2, ia2, ja2, resd, 1, 2, 3, gh, im, jm, 2 * nb, cd, 2e-16, 1]),
        ("bcg_computejacobianfromdz", [jac, ia, ja, resd, 4, 0, 6, gh, im, jm, nb]),
        ("bcg_compute_norml2", [n2, m2, res, im, jm, gh]),
        ("bcg_compute_norml2inf", [n3, m3, res, im, jm, gh]),
        ("bcg_compute_maxnorm", [n4, i4, j4, res, im, jm, gh]),
        ("bcg_computegeom_2d", geo + [im, jm, gh]),
        ("bcg_initblfv", [ph["muinf"], g["xc"], g["yc"], c["w"], c["field"], im, gh, jm]),
        ("bcg_set_bndbl_2d", [c["w"], c["field"], c["wbd"], im, jm, gh]),
        ("bcg_impli_matrix_free_2d", [dwi, g["nx"], g["ny"], c["w"], res, g["vol"], g["volf"], 1.0, 5.0, ph["gam"],
                                      ph["rgaz"], ph["prandtl"], 10, gh, ph["cv"], ph["cs"], ph["muref"],
                                      ph["tref"], ph["cs"], im, jm, 5]),
    ])


def test_in_place_arguments_must_be_fortran_float64(recorder):
    """As with f2py, an intent(inout) array that is not a Fortran-ordered
    float64 array is refused rather than silently copied."""
    c, g, ph, z = _bl()
    it = c["interf"]
    with pytest.raises(ValueError):
        f_bnd.bc_extrapolate_o2_2d(np.ascontiguousarray(c["w"]), "Ihi", it["Ihi"], g["im"], g["jm"], g["gh"])
    with pytest.raises(ValueError):
        f_misc.testvector(np.zeros(c["w"].shape, np.float32, order="F"), 0, 0, 0, g["gh"])
    assert recorder == []
