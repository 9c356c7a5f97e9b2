"""Shared test helpers: case construction and boundary sequences through the
oracle (the checker) and through the library (the product)."""
import numpy as np

from broadcast_gb300 import cases
from oracle import oracle as O

GH = cases.GH


class OracleOps:
    computegeom = staticmethod(O.computegeom)
    initblfv = staticmethod(O.initblfv)
    set_bndbl = staticmethod(O.set_bndbl)


def bl_case(im=40, jm=30, **kw):
    return cases.bl_case(im, jm, ops=OracleOps, **kw)


def cyl_case(im=28, jm=20, **kw):
    return cases.cyl_case(im, jm, ops=OracleOps, **kw)


# --- boundary sequences in the reference drivers' order --------------------------
def oracle_bcs(c, w, wd=None):
    """BL: BROADCAST_npz.py:1018-1021 (primal) / :1079-1082 (tangent);
    cylinder: handleBC.applyBC order [Jhi, Jlo, Ilo, Ihi] (handleBC.sortBC)."""
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    if c["kind"] == "bl":
        O.bc_inlet(w, "Ilo", it["Ilo"], c["field"], g["nx"], g["ny"], ph["gam"], im, jm, gh, wd=wd)
        O.bc_noref(w, c["wbd"], "Jhi", it["Jhi"], g["nx"], g["ny"], ph["gam"], gh, im, jm, wd=wd)
        O.bc_extrap(w, "Ihi", it["Ihi"], im, jm, gh, wd=wd)
        O.bc_wall(w, "Jlo", ph["gam"], it["Jlo"], gh, im, jm, wd=wd)
    else:
        O.bc_noref(w, c["wbd"], "Jhi", it["Jhi"], g["nx"], g["ny"], ph["gam"], gh, im, jm, wd=wd)
        O.bc_wall(w, "Jlo", ph["gam"], it["Jlo"], gh, im, jm, wd=wd)
        for _ in range(2):  # interf3 and interf4 each apply both copies
            for arr in ([w] if wd is None else [wd, w]):
                O.jn_match(arr, it["prr1"], (gh,) * 4, im, jm, arr, it["prd2"], (gh,) * 4, im, jm, it["tr"], 5)
                O.jn_match(arr, it["prr2"], (gh,) * 4, im, jm, arr, it["prd1"], (gh,) * 4, im, jm, it["tr"], 5)


def lib_bcs(c, w, wd=None):
    """The same sequences through the drop-in modules (numpy or torch arrays)."""
    from broadcast_gb300.srcfv import f_bnd, f_lin
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    nx, ny = c.get("nx_dev", g["nx"]), c.get("ny_dev", g["ny"])
    if c["kind"] == "bl":
        if wd is None:
            f_bnd.bc_supandsubinlet_2d(w, "Ilo", it["Ilo"], c["field"], nx, ny, ph["gam"], im, jm)
            f_bnd.bc_no_reflexion_2d(w, c["wbd"], "Jhi", it["Jhi"], nx, ny, ph["gam"], gh, im, jm)
            f_bnd.bc_extrapolate_o2_2d(w, "Ihi", it["Ihi"], im, jm, gh)
            f_bnd.bc_wall_viscous_adia_2d(w, "Jlo", ph["gam"], it["Jlo"], gh, im, jm)
        else:
            f_lin.bc_supandsubinlet_2d_d(w, wd, "Ilo", it["Ilo"], c["field"], nx, ny, ph["gam"], im, jm)
            f_lin.bc_no_reflexion_2d_d(w, wd, c["wbd"], "Jhi", it["Jhi"], nx, ny, ph["gam"], gh, im, jm)
            f_lin.bc_extrapolate_o2_2d_d(w, wd, "Ihi", it["Ihi"], im, jm, gh)
            f_lin.bc_wall_viscous_adia_2d_d(w, wd, "Jlo", ph["gam"], it["Jlo"], gh, im, jm)
    else:
        if wd is None:
            f_bnd.bc_no_reflexion_2d(w, c["wbd"], "Jhi", it["Jhi"], nx, ny, ph["gam"], gh, im, jm)
            f_bnd.bc_wall_viscous_adia_2d(w, "Jlo", ph["gam"], it["Jlo"], gh, im, jm)
        else:
            f_lin.bc_no_reflexion_2d_d(w, wd, c["wbd"], "Jhi", it["Jhi"], nx, ny, ph["gam"], gh, im, jm)
            f_lin.bc_wall_viscous_adia_2d_d(w, wd, "Jlo", ph["gam"], it["Jlo"], gh, im, jm)
        for _ in range(2):
            for arr in ([w] if wd is None else [wd, w]):
                f_bnd.jn_match_2d(arr, it["prr1"], gh, gh, gh, gh, im, jm, arr, it["prd2"], gh, gh, gh, gh, im, jm,
                                  it["tr"])
                f_bnd.jn_match_2d(arr, it["prr2"], gh, gh, gh, gh, im, jm, arr, it["prd1"], gh, gh, gh, gh, im, jm,
                                  it["tr"])


def flux_scale(c, w):
    """Per-variable flux magnitude: max over cells of (|f_e| + |g_e|) times the
    largest face length -- the scale of the face fluxes the residual differences."""
    g, ph = c["grid"], c["phys"]
    ro = w[..., 0]
    u, v = w[..., 1] / ro, w[..., 2] / ro
    p = (ph["gam"] - 1.0) * (w[..., 4] - 0.5 * ro * (u * u + v * v + (w[..., 3] / ro) ** 2))
    f = np.stack([w[..., 1], w[..., 1] * u + p, w[..., 1] * v, w[..., 1] * w[..., 3] / ro, (w[..., 4] + p) * u], -1)
    gg = np.stack([w[..., 2], w[..., 2] * u, w[..., 2] * v + p, w[..., 2] * w[..., 3] / ro, (w[..., 4] + p) * v], -1)
    sn = np.sqrt(g["nx"] ** 2 + g["ny"] ** 2).max()
    return (np.abs(f) + np.abs(gg)).reshape(-1, 5).max(0) * sn


def interior(a, gh=GH):
    return a[gh:-gh, gh:-gh, ...]


def rel_err(a, b, scale, gh=GH):
    """max-norm error per variable scaled by `scale` (5-vector); returns the max."""
    d = np.abs(interior(a, gh) - interior(b, gh)).reshape(-1, 5).max(0)
    return float((d / scale).max())
