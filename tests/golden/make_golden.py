"""Generate the golden fixtures of tests/golden/ from the reference's own
routines (oracle/_ref/libref.so, built by `python oracle/ref_build.py` from a
reference checkout; see oracle/ref_translate.py).

    python tests/golden/make_golden.py

Each fixture holds the inputs (grid metrics, state, directions) and the
reference outputs of one small case, so that the oracle and the CUDA path can
be checked against the reference where the reference is not available.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from broadcast_gb300 import cases  # noqa: E402
from oracle import ref  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
PHYS = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")


class RefOps:
    @staticmethod
    def computegeom(x0, y0, nx, ny, xc, yc, vol, volf, im, jm, gh):
        ref.call("computegeom_2d", x0, y0, nx, ny, xc, yc, vol, volf, im, jm, gh)

    @staticmethod
    def initblfv(muinf, xc, yc, w, field, im, gh, jm):
        ref.call("initblfv", muinf, xc, yc, w, field, im, gh, jm)

    @staticmethod
    def set_bndbl(w, field, wbd, im, jm, gh):
        ref.call("set_bndbl_2d", w, field, wbd, im, jm, gh)


def fi(a):
    return np.asfortranarray(np.asarray(a, dtype=np.int32))


def ref_bcs(c, w, wd=None):
    """The drivers' boundary sequences through the reference routines."""
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    gam = ph["gam"]
    if c["kind"] == "bl":
        fld, wbd = c["field"], c["wbd"]
        lm_f, lm_b = fld.shape[0], wbd.shape[0]
        if wd is None:
            ref.call("bc_supandsubinlet_2d", w, "Ilo", fi(it["Ilo"]), fld, g["nx"], g["ny"], gam, im, jm, lm_f, gh)
            ref.call("bc_no_reflexion_2d", w, wbd, "Jhi", fi(it["Jhi"]), g["nx"], g["ny"], gam, gh, im, jm, lm_b)
            ref.call("bc_extrapolate_o2_2d", w, "Ihi", fi(it["Ihi"]), im, jm, gh, 5)
            ref.call("bc_wall_viscous_adia_2d", w, "Jlo", gam, fi(it["Jlo"]), gh, im, jm)
        else:
            ref.call("bc_supandsubinlet_2d_d", w, wd, "Ilo", fi(it["Ilo"]), fld, g["nx"], g["ny"], gam, im, jm, lm_f, gh)
            ref.call("bc_no_reflexion_2d_d", w, wd, wbd, "Jhi", fi(it["Jhi"]), g["nx"], g["ny"], gam, gh, im, jm, lm_b)
            ref.call("bc_extrapolate_o2_2d_d", w, wd, "Ihi", fi(it["Ihi"]), im, jm, gh, 5)
            ref.call("bc_wall_viscous_adia_2d_d", w, wd, "Jlo", gam, fi(it["Jlo"]), gh, im, jm)
    else:
        wbd = c["wbd"]
        if wd is None:
            ref.call("bc_no_reflexion_2d", w, wbd, "Jhi", fi(it["Jhi"]), g["nx"], g["ny"], gam, gh, im, jm, wbd.shape[0])
            ref.call("bc_wall_viscous_adia_2d", w, "Jlo", gam, fi(it["Jlo"]), gh, im, jm)
        else:
            ref.call("bc_no_reflexion_2d_d", w, wd, wbd, "Jhi", fi(it["Jhi"]), g["nx"], g["ny"], gam, gh, im, jm,
                     wbd.shape[0])
            ref.call("bc_wall_viscous_adia_2d_d", w, wd, "Jlo", gam, fi(it["Jlo"]), gh, im, jm)
        # periodic joins through the reference's jn_match_2d (borders/jn_match.F90), the
        # drivers' ranges (cylinder.py:481-486), each array its own donor
        for a in ([w] if wd is None else [wd, w]):
            for prr, prd in ((it["prr1"], it["prd2"]), (it["prr2"], it["prd1"])):
                ref.call("jn_match_2d", a, fi(prr), gh, gh, gh, gh, im, jm, a, fi(prd), gh, gh, gh, gh, im, jm,
                         fi(it["tr"]), 5)


def residual_args(c):
    g, ph = c["grid"], c["phys"]
    return (g["x0"], g["y0"], g["nx"], g["ny"], g["xc"], g["yc"], g["vol"], g["volf"], g["gh"]) + tuple(
        ph[k] for k in PHYS) + (g["im"], g["jm"])


def make(kind, im, jm, seed):
    c = cases.bl_case(im, jm, seed=seed, ops=RefOps) if kind == "bl" else cases.cyl_case(im, jm, seed=seed, ops=RefOps)
    g, ph = c["grid"], c["phys"]
    w_raw = c["w"].copy(order="F")
    w = c["w"]
    ref_bcs(c, w)
    rng = np.random.default_rng(seed + 100)
    out = {"kind": kind, "im": im, "jm": jm, "gh": g["gh"], "w_raw": w_raw, "w": w.copy(order="F")}
    for k in ("x0", "y0", "nx", "ny", "xc", "yc", "vol", "volf"):
        out[k] = g[k]
    for k in PHYS:
        out["phys_" + k] = ph[k]
    if kind == "bl":
        out["field"], out["wbd"] = c["field"], c["wbd"]
    else:
        out["wbd"] = c["wbd"]
    res = np.zeros_like(w)
    ref.call("flux_num_dnc5_2d", res, w, *residual_args(c))
    out["res"] = res
    # tangent: two directions, ghosts filled by the linearised boundary sequence
    wds, resds = [], []
    for d in range(2):
        wd = np.zeros_like(w)
        wd[3:-3, 3:-3] = rng.standard_normal((im, jm, 5))
        wtmp = w.copy(order="F")
        ref_bcs(c, wtmp, wd)
        r, rd = np.zeros_like(w), np.zeros_like(w)
        ref.call("flux_num_dnc5_2d_d", r, rd, w, wd, *residual_args(c))
        wds.append(wd)
        resds.append(rd)
    out["wd"] = np.stack(wds)
    out["resd"] = np.stack(resds)
    # the scheme without the wall rows (flux_num_dnc5_nowall_2d and its tangent) on the same state
    res_nw = np.zeros_like(w)
    ref.call("flux_num_dnc5_nowall_2d", res_nw, w, *residual_args(c))
    r_nw, rd_nw = np.zeros_like(w), np.zeros_like(w)
    ref.call("flux_num_dnc5_nowall_2d_d", r_nw, rd_nw, w, wds[0], *residual_args(c))
    out["res_nowall"], out["resd_nowall"] = res_nw, rd_nw
    # spanwise operators applied to the first direction (coeffs_5p_dz, coeffs_5p_dz2)
    span_args = residual_args(c)[:9] + tuple(ph[k] for k in PHYS[:9]) + (im, jm)
    for name, key in (("coeffs_5p_dz", "dz"), ("coeffs_5p_dz2", "dzz")):
        o = np.zeros_like(w)
        ref.call(name, o, w, wds[0], *span_args)
        out[key] = o
    # adjoint: one cotangent on the interior
    rb = np.zeros_like(w)
    rb[3:-3, 3:-3] = rng.standard_normal((im, jm, 5))
    out["rb"] = rb.copy(order="F")
    wb, r3 = np.zeros_like(w), np.zeros_like(w)
    ref.call("flux_num_dnc5_2d_b", r3, rb, w, wb, *residual_args(c))
    out["wb"] = wb
    # adjoints of the ghost fills (adjoint/bc_*_b.f90), each applied to a
    # random cotangent on the state just before that fill in the driver chain
    it = c["interf"]
    gam, gh = ph["gam"], g["gh"]
    wst = w_raw.copy(order="F")
    chain = [("inlet", "Ilo"), ("noref", "Jhi"), ("extrap", "Ihi"), ("wall", "Jlo")] if kind == "bl" else \
        [("noref", "Jhi"), ("wall", "Jlo")]
    for bk, loc in chain:
        wb0 = np.asfortranarray(rng.standard_normal(w.shape))
        wb = wb0.copy(order="F")
        wcopy = wst.copy(order="F")
        if bk == "inlet":
            fld = c["field"]
            ref.call("bc_supandsubinlet_2d_b", wcopy, wb, loc, fi(it[loc]), fld, g["nx"], g["ny"], gam, im, jm,
                     fld.shape[0], gh)
            ref.call("bc_supandsubinlet_2d", wst, loc, fi(it[loc]), fld, g["nx"], g["ny"], gam, im, jm, fld.shape[0], gh)
        elif bk == "noref":
            wbd = c["wbd"]
            ref.call("bc_no_reflexion_2d_b", wcopy, wb, wbd, loc, fi(it[loc]), g["nx"], g["ny"], gam, gh, im, jm,
                     wbd.shape[0])
            ref.call("bc_no_reflexion_2d", wst, wbd, loc, fi(it[loc]), g["nx"], g["ny"], gam, gh, im, jm, wbd.shape[0])
        elif bk == "extrap":
            ref.call("bc_extrapolate_o2_2d_b", wcopy, wb, loc, fi(it[loc]), im, jm, gh, 5)
            ref.call("bc_extrapolate_o2_2d", wst, loc, fi(it[loc]), im, jm, gh, 5)
        else:
            ref.call("bc_wall_viscous_adia_2d_b", wcopy, wb, loc, gam, fi(it[loc]), gh, im, jm)
            ref.call("bc_wall_viscous_adia_2d", wst, loc, gam, fi(it[loc]), gh, im, jm)
        out["bcb_%s_w" % bk] = wcopy
        out["bcb_%s_in" % bk] = wb0
        out["bcb_%s_out" % bk] = wb
    if kind == "cyl":
        # adjoint of one periodic join copy (adjoint/jn_match_2d_b.f90)
        wrb0 = np.asfortranarray(rng.standard_normal(w.shape))
        wrb, wdb = wrb0.copy(order="F"), np.asfortranarray(rng.standard_normal(w.shape))
        ref.call("jn_match_2d_b", w.copy(order="F"), wrb, fi(it["prr1"]), gh, gh, gh, gh, im, jm, w.copy(order="F"),
                 wdb, fi(it["prd2"]), gh, gh, gh, gh, im, jm, fi(it["tr"]), 5)
        out.update(jnb_wrb_in=wrb0, jnb_wrb_out=wrb, jnb_wdb_out=wdb)
    # norms of the residual
    n2, nm = np.zeros(5), np.zeros(5)
    ref.call("compute_norml2", n2, nm, res, im, jm, 3)
    ni2, ninf = np.zeros(5), np.zeros(5)
    ref.call("compute_norml2inf", ni2, ninf, res, im, jm, 3)
    mx, imx, jmx = np.zeros(5), np.zeros(5, np.int32), np.zeros(5, np.int32)
    ref.call("compute_maxnorm", mx, imx, jmx, res, im, jm, 3)
    out.update(norml2=n2, nmoy=nm, ninf=ninf, maxnorm=mx, imax=imx, jmax=jmx)
    return out


def make_indexing(im=16, jm=11, gh=3, seed=7):
    rng = np.random.default_rng(seed)
    resd = np.asfortranarray(rng.standard_normal((im + 2 * gh, jm + 2 * gh, 5)))
    coef = np.asfortranarray(rng.standard_normal((im, jm)))
    nb = im * jm * 49 * 25
    out = {"im": im, "jm": jm, "gh": gh, "resd": resd, "coefdiag": coef}
    seeds = [(0, 0, 0), (2, 5, 1), (4, 6, 6), (1, 3, 4)]
    for name in ("computejacobianfromjv", "computejacobianfromjv_relaxed", "computejacobianfromjv_relaxed_withjn",
                 "computejacobianfromjv_withjn", "computejacobianfromdz"):
        jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
        for (m, l, k) in seeds:
            if "relaxed" in name:
                ref.call(name, jac, ia, ja, resd, m, l, k, gh, im, jm, nb, coef)
            else:
                ref.call(name, jac, ia, ja, resd, m, l, k, gh, im, jm, nb)
        out[name + "_jac"], out[name + "_ia"], out[name + "_ja"] = jac, ia, ja
    # the two-zone check variant: zone 0 then zone 1 into the same arrays
    nb2 = nb * 2
    jac, ia, ja = np.zeros(nb2), np.zeros(nb2, np.int32), np.zeros(nb2, np.int32)
    for n in (0, 1):
        for (m, l, k) in seeds:
            ref.call("computejacobianfromjv_relaxed_withjnandcheck", jac, ia, ja, resd, m, l, k, gh, im, jm, nb2, coef,
                     2e-16, n)
    out["check_jac"], out["check_ia"], out["check_ja"] = jac, ia, ja
    tv = []
    for (m, l, k) in seeds:
        wd = np.zeros((im + 2 * gh, jm + 2 * gh, 5), order="F")
        ref.call("testvector", wd, m, l, k, gh, im, jm)
        tv.append(wd)
        wd = np.zeros((im + 2 * gh, jm + 2 * gh, 5), order="F")
        ref.call("testvector_partial", wd, m, l, k, gh, im, jm, 2, im - 2, 0, jm - 1)
        tv.append(wd)
    out["testvectors"] = np.stack(tv)
    out["seeds"] = np.array(seeds, dtype=np.int32)
    return out


SCHEMES = {"dnc%d_%s_12x11" % (o, k): (o, k) for o in (3, 7, 9) for k in ("bl", "cyl")}


def make_scheme(order, kind, im=12, jm=11, seed=11):
    """flux_num_dnc{order}_2d, its tangent and the _nowall pair on one small
    case with the driver's ghost width gh = (order+1)//2: the boundary layer
    with k2 = 1.01 (sensor on) or the cylinder with k2 = 0."""
    gh = (order + 1) // 2
    c = cases.bl_case(im, jm, seed=seed, ops=RefOps, gh=gh) if kind == "bl" else \
        cases.cyl_case(im, jm, seed=seed, ops=RefOps, gh=gh)
    g, ph = c["grid"], c["phys"]
    w = c["w"]
    ref_bcs(c, w)
    rng = np.random.default_rng(seed + 100)
    out = {"kind": kind, "order": order, "im": im, "jm": jm, "gh": gh, "w": w.copy(order="F")}
    for k in ("x0", "y0", "nx", "ny", "xc", "yc", "vol", "volf"):
        out[k] = g[k]
    for k in PHYS:
        out["phys_" + k] = ph[k]
    out["wbd"] = c["wbd"]
    if kind == "bl":
        out["field"] = c["field"]
    wd = np.zeros_like(w)
    wd[gh:-gh, gh:-gh] = rng.standard_normal((im, jm, 5))
    ref_bcs(c, w.copy(order="F"), wd)
    out["wd"] = wd
    for suffix in ("", "_nowall"):
        name = "flux_num_dnc%d%s_2d" % (order, suffix)
        res = np.zeros_like(w)
        ref.call(name, res, w, *residual_args(c))
        r, rd = np.zeros_like(w), np.zeros_like(w)
        ref.call(name + "_d", r, rd, w, wd, *residual_args(c))
        out["res" + suffix], out["resd" + suffix] = res, rd
    return out


def make_impli(kind, im, jm, seed, lmaxes=(1, 2, 10), dtcoef=1.0, cfl=5.0):
    """impli_matrix_free_2d on the residual of a small case, as the 'impli' time
    marching calls it (BROADCAST_npz.py:941, s_suth = cs)."""
    c = cases.bl_case(im, jm, seed=seed, ops=RefOps) if kind == "bl" else cases.cyl_case(im, jm, seed=seed, ops=RefOps)
    g, ph = c["grid"], c["phys"]
    w = c["w"]
    ref_bcs(c, w)
    res = np.zeros_like(w)
    ref.call("flux_num_dnc5_2d", res, w, *residual_args(c))
    out = {"kind": kind, "im": im, "jm": jm, "gh": g["gh"], "w": w.copy(order="F"), "dw": res, "dtcoef": dtcoef,
           "cfl": cfl, "lmax": np.array(lmaxes, dtype=np.int32), "wbd": c["wbd"]}
    if kind == "bl":
        out["field"] = c["field"]
    for k in ("x0", "y0", "nx", "ny", "xc", "yc", "vol", "volf"):
        out[k] = g[k]
    for k in PHYS:
        out["phys_" + k] = ph[k]
    for lm in lmaxes:
        dwi = np.full_like(w, 3.0)
        ref.call("impli_matrix_free_2d", dwi, g["nx"], g["ny"], w, res, g["vol"], g["volf"], dtcoef, cfl, ph["gam"],
                 ph["rgaz"], ph["prandtl"], int(lm), g["gh"], ph["cv"], ph["cs"], ph["muref"], ph["tref"], ph["cs"], im,
                 jm, 5)
        out["dwi_%d" % lm] = dwi
    return out


def make_nowall_adjoint(kind, im, jm, seed):
    """flux_num_dnc5_nowall_2d_b (the reference's Tapenade adjoint of the scheme
    without the wall rows) for one random cotangent."""
    c = cases.bl_case(im, jm, seed=seed, ops=RefOps) if kind == "bl" else cases.cyl_case(im, jm, seed=seed, ops=RefOps)
    g, ph = c["grid"], c["phys"]
    w = c["w"]
    ref_bcs(c, w)
    rng = np.random.default_rng(seed + 100)
    rb = np.zeros_like(w)
    rb[3:-3, 3:-3] = rng.standard_normal((im, jm, 5))
    out = {"kind": kind, "im": im, "jm": jm, "gh": g["gh"], "w": w.copy(order="F"), "rb": rb.copy(order="F"),
           "wbd": c["wbd"]}
    if kind == "bl":
        out["field"] = c["field"]
    for k in ("x0", "y0", "nx", "ny", "xc", "yc", "vol", "volf"):
        out[k] = g[k]
    for k in PHYS:
        out["phys_" + k] = ph[k]
    wb = np.zeros_like(w)
    ref.call("flux_num_dnc5_nowall_2d_b", np.zeros_like(w), rb.copy(order="F"), w, wb, *residual_args(c))
    out["wb_nowall"] = wb
    return out


NOWALL_ADJ = {"adj_nowall_bl_16x12": ("bl", 16, 12, 12), "adj_nowall_cyl_16x12": ("cyl", 16, 12, 13)}


IMPLI = {"impli_bl_16x10": ("bl", 16, 10, 5), "impli_cyl_14x8": ("cyl", 14, 8, 6)}


def main():
    if not ref.available():
        raise SystemExit("oracle/_ref is not built: run python oracle/ref_build.py first")
    for name, (kind, im, jm, seed) in {"bl_14x10": ("bl", 14, 10, 0), "cyl_14x8": ("cyl", 14, 8, 1),
                                       "bl_23x17": ("bl", 23, 17, 3)}.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **make(kind, im, jm, seed))
    np.savez_compressed(os.path.join(HERE, "indexing_16x11.npz"), **make_indexing())
    for name, (order, kind) in SCHEMES.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **make_scheme(order, kind))
    for name, args in IMPLI.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **make_impli(*args))
    for name, args in NOWALL_ADJ.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **make_nowall_adjoint(*args))
    print("written:", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))


if __name__ == "__main__":
    main()
