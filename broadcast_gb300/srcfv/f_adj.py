"""Drop-in for the reference's srcfv.f_adj (Tapenade reverse-mode routines).

flux_num_dnc5_2d_b       : adjoint/flux_num_dnc5_b.f90:15 -- wb = (dR/dw)^T residub
                           on every padded cell (wb overwritten); the interior
                           of residub is zeroed.
flux_num_dnc5_nowall_2d_b: adjoint/flux_num_dnc5_nowall_b.f90 -- the same for the
                           scheme without the wall rows.
bc_wall_viscous_adia_2d_b: adjoint/bc_wall_viscous_b.f90:11
bc_no_reflexion_2d_b     : adjoint/bc_no_reflexion_b.f90:16
bc_supandsubinlet_2d_b   : adjoint/bc_supandsubinlet_b.f90:11
bc_extrapolate_o2_2d_b   : adjoint/bc_extrapolateo2_b.f90:18
jn_match_2d_b            : adjoint/jn_match_2d_b.f90:1
The fill adjoints add J^T wb(ghosts) to wb on the cells each fill reads and
zero wb on the ghosts it writes; w is left as it is.
"""
import numpy as np

from .._f2py import arr, call, dims_from_cell, interf4, shape
from .f_bnd import _loc, _pr


def flux_num_dnc5_2d_b(residu, residub, w, wb, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs,
                       muref, tref, s_suth, k2, k4, im=None, jm=None):
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    call("bcg_flux_num_dnc5_2d_b", None, arr(residub, "residub", True), arr(w, "w"), arr(wb, "wb", True), None, None,
         arr(nx, "nx"), arr(ny, "ny"), None, None, arr(vol, "vol"), arr(volf, "volf"), gh, cp, cv, prandtl, gam, rgaz,
         cs, muref, tref, s_suth, k2, k4, int(im), int(jm))


def flux_num_dnc5_nowall_2d_b(residu, residub, w, wb, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam,
                              rgaz, cs, muref, tref, s_suth, k2, k4, im=None, jm=None):
    """adjoint/flux_num_dnc5_nowall_b.f90: the adjoint of the scheme without the wall rows."""
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    call("bcg_flux_num_dnc5_nowall_2d_b", None, arr(residub, "residub", True), arr(w, "w"), arr(wb, "wb", True), None,
         None, arr(nx, "nx"), arr(ny, "ny"), None, None, arr(vol, "vol"), arr(volf, "volf"), gh, cp, cv, prandtl, gam,
         rgaz, cs, muref, tref, s_suth, k2, k4, int(im), int(jm))


def bc_wall_viscous_adia_2d_b(w, wb, loc, gam, interf, gh, im=None, jm=None):
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    call("bcg_bc_wall_viscous_adia_2d_b", arr(w, "w"), arr(wb, "wb", True), _loc(loc), gam, interf4(interf), gh,
         int(im), int(jm))


def bc_no_reflexion_2d_b(w, wb, wbd, loc, interf, nx, ny, gam, gh, im=None, jm=None, lm=None):
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    wbd = arr(wbd, "wbd")
    lm = shape(wbd)[0] if lm is None else lm
    call("bcg_bc_no_reflexion_2d_b", arr(w, "w"), arr(wb, "wb", True), wbd, _loc(loc), interf4(interf),
         arr(nx, "nx"), arr(ny, "ny"), gam, gh, int(im), int(jm), int(lm))


def bc_supandsubinlet_2d_b(w, wb, loc, interf, field, nx, ny, gam, im, jm, lm=None, gh=None):
    field = arr(field, "field")
    gh = shape(field)[1] if gh is None else int(gh)
    lm = shape(field)[0] if lm is None else lm
    call("bcg_bc_supandsubinlet_2d_b", arr(w, "w"), arr(wb, "wb", True), _loc(loc), interf4(interf), field,
         arr(nx, "nx"), arr(ny, "ny"), gam, int(im), int(jm), int(lm), gh)


def bc_extrapolate_o2_2d_b(w, wb, loc, interf, im, jm, gh, em=None):
    em = shape(w)[2] if em is None else em
    call("bcg_bc_extrapolate_o2_2d_b", arr(w, "w"), arr(wb, "wb", True), _loc(loc), interf4(interf), int(im),
         int(jm), int(gh), int(em))


def jn_match_2d_b(wr, wrb, prr, gh1r, gh2r, gh3r, gh4r, imr, jmr, wd, wdb, prd, gh1d, gh2d, gh3d, gh4d, imd, jmd, tr,
                  em=None):
    em = shape(wrb)[2] if em is None else em
    t = np.ascontiguousarray(np.asarray(tr, dtype=np.int32).ravel())
    call("bcg_jn_match_2d_b", None, arr(wrb, "wrb", True), _pr(prr), int(gh1r), int(gh2r), int(gh3r), int(gh4r),
         int(imr), int(jmr), None, arr(wdb, "wdb", True), _pr(prd), int(gh1d), int(gh2d), int(gh3d), int(gh4d),
         int(imd), int(jmd), t, int(em))
