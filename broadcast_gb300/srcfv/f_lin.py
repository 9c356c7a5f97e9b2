"""Drop-in for the reference's srcfv.f_lin (Tapenade tangent routines).

flux_num_dnc5_2d_d       : tangent/flux_num_dnc5_d.f90:15
flux_num_dnc5_nowall_2d_d: tangent/flux_num_dnc5_nowall_d.f90
flux_num_dnc{3,7,9}[_nowall]_2d_d: tangent/flux_num_dnc{3,7,9}[_nowall]_d.f90
bc_wall_viscous_adia_2d_d: tangent/bc_wall_viscous_d.f90:11
bc_no_reflexion_2d_d     : tangent/bc_no_reflexion_d.f90:16
bc_supandsubinlet_2d_d   : tangent/bc_supandsubinlet_d.f90:11
bc_extrapolate_o2_2d_d   : tangent/bc_extrapolateo2_d.f90:18
jn_match_2d_d            : tangent/jn_match_2d_d.f90:11
Each routine updates both the state and its tangent, as the Tapenade code does.
"""
import numpy as np

from .._f2py import arr, call, dims_from_cell, interf4, shape
from .f_bnd import _loc


def flux_num_dnc5_2d_d(residu, residud, w, wd, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs,
                       muref, tref, s_suth, k2, k4, im=None, jm=None):
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    call("bcg_flux_num_dnc5_2d_d", arr(residu, "residu", True), arr(residud, "residud", True), arr(w, "w"),
         arr(wd, "wd"), None, None, arr(nx, "nx"), arr(ny, "ny"), None, None, arr(vol, "vol"), arr(volf, "volf"), gh,
         cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4, int(im), int(jm))


def flux_num_dnc5_nowall_2d_d(residu, residud, w, wd, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam,
                              rgaz, cs, muref, tref, s_suth, k2, k4, im=None, jm=None):
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    call("bcg_flux_num_dnc5_nowall_2d_d", arr(residu, "residu", True), arr(residud, "residud", True), arr(w, "w"),
         arr(wd, "wd"), None, None, arr(nx, "nx"), arr(ny, "ny"), None, None, arr(vol, "vol"), arr(volf, "volf"), gh,
         cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, k2, k4, int(im), int(jm))


def _scheme_d(symbol):
    def tangent(residu, residud, w, wd, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref,
                tref, s_suth, k2, k4, im=None, jm=None):
        gh = int(gh)
        if im is None or jm is None:
            im, jm = dims_from_cell(w, gh)
        call(symbol, arr(residu, "residu", True), arr(residud, "residud", True), arr(w, "w"), arr(wd, "wd"), None, None,
             arr(nx, "nx"), arr(ny, "ny"), None, None, arr(vol, "vol"), arr(volf, "volf"), gh, cp, cv, prandtl, gam,
             rgaz, cs, muref, tref, s_suth, k2, k4, int(im), int(jm))
    tangent.__name__ = symbol[4:]
    tangent.__doc__ = "Residual and tangent of the DNC scheme (srcfv/tangent/%s.f90)." % symbol[4:-3]
    return tangent


flux_num_dnc3_2d_d = _scheme_d("bcg_flux_num_dnc3_2d_d")
flux_num_dnc7_2d_d = _scheme_d("bcg_flux_num_dnc7_2d_d")
flux_num_dnc9_2d_d = _scheme_d("bcg_flux_num_dnc9_2d_d")
flux_num_dnc3_nowall_2d_d = _scheme_d("bcg_flux_num_dnc3_nowall_2d_d")
flux_num_dnc7_nowall_2d_d = _scheme_d("bcg_flux_num_dnc7_nowall_2d_d")
flux_num_dnc9_nowall_2d_d = _scheme_d("bcg_flux_num_dnc9_nowall_2d_d")


def bc_wall_viscous_adia_2d_d(w, wd, loc, gam, interf, gh, im=None, jm=None):
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    call("bcg_bc_wall_viscous_adia_2d_d", arr(w, "w", True), arr(wd, "wd", True), _loc(loc), gam, interf4(interf), gh,
         int(im), int(jm))


def bc_no_reflexion_2d_d(w, wd, wbd, loc, interf, nx, ny, gam, gh, im=None, jm=None, lm=None):
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    wbd = arr(wbd, "wbd")
    lm = shape(wbd)[0] if lm is None else lm
    call("bcg_bc_no_reflexion_2d_d", arr(w, "w", True), arr(wd, "wd", True), wbd, _loc(loc), interf4(interf),
         arr(nx, "nx"), arr(ny, "ny"), gam, gh, int(im), int(jm), int(lm))


def bc_supandsubinlet_2d_d(w, wd, loc, interf, field, nx, ny, gam, im, jm, gh=None, lm=None):
    field = arr(field, "field")
    gh = shape(field)[1] if gh is None else int(gh)
    lm = shape(field)[0] if lm is None else lm
    call("bcg_bc_supandsubinlet_2d_d", arr(w, "w", True), arr(wd, "wd", True), _loc(loc), interf4(interf), field,
         arr(nx, "nx"), arr(ny, "ny"), gam, int(im), int(jm), int(lm), gh)


def bc_extrapolate_o2_2d_d(w, wd, loc, interf, im, jm, gh, em=None):
    em = shape(w)[2] if em is None else em
    call("bcg_bc_extrapolate_o2_2d_d", arr(w, "w", True), arr(wd, "wd", True), _loc(loc), interf4(interf), int(im),
         int(jm), int(gh), int(em))


def jn_match_2d_d(wr, wrd, prr, gh1r, gh2r, gh3r, gh4r, imr, jmr, wd, wdd, prd, gh1d, gh2d, gh3d, gh4d, imd, jmd, tr,
                  em=None):
    em = shape(wr)[2] if em is None else em
    t = np.ascontiguousarray(np.asarray(tr, dtype=np.int32).ravel())
    call("bcg_jn_match_2d_d", arr(wr, "wr", True), arr(wrd, "wrd", True), interf4(prr), gh1r, gh2r, gh3r, gh4r, imr,
         jmr, arr(wd, "wd"), arr(wdd, "wdd"), interf4(prd), gh1d, gh2d, gh3d, gh4d, imd, jmd, t, int(em))
