"""Drop-in for the reference's srcfv.f_bnd (ghost-cell boundary fills).

bc_wall_viscous_adia_2d : borders/bc_wall_viscous.F90:2
bc_no_reflexion_2d      : borders/bc_no_reflexion.F90:8
bc_supandsubinlet_2d    : borders/bc_supandsubinlet.F90:2
bc_extrapolate_o2_2d    : borders/bc_extrapolate.F90:39
jn_match_2d             : borders/jn_match.F90:3
jn_match_geom_2d        : borders/jn_match_geom.F90:7
"""
import numpy as np

from .._f2py import arr, call, dims_from_cell, interf4, shape


def _loc(loc):
    return loc.encode() if isinstance(loc, str) else loc


def bc_wall_viscous_adia_2d(w, loc, gam, interf, gh, im=None, jm=None):
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    call("bcg_bc_wall_viscous_adia_2d", arr(w, "w", True), _loc(loc), gam, interf4(interf), gh, int(im), int(jm))


def bc_no_reflexion_2d(w, wbd, loc, interf, nx, ny, gam, gh, im=None, jm=None, lm=None):
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    wbd = arr(wbd, "wbd")
    lm = shape(wbd)[0] if lm is None else lm
    call("bcg_bc_no_reflexion_2d", arr(w, "w", True), wbd, _loc(loc), interf4(interf), arr(nx, "nx"), arr(ny, "ny"),
         gam, gh, int(im), int(jm), int(lm))


def bc_supandsubinlet_2d(w, loc, interf, field, nx, ny, gam, im, jm, gh=None, lm=None):
    field = arr(field, "field")
    gh = shape(field)[1] if gh is None else int(gh)
    lm = shape(field)[0] if lm is None else lm
    call("bcg_bc_supandsubinlet_2d", arr(w, "w", True), _loc(loc), interf4(interf), field, arr(nx, "nx"),
         arr(ny, "ny"), gam, int(im), int(jm), int(lm), gh)


def bc_extrapolate_o2_2d(w, loc, interf, im, jm, gh, em=None):
    em = shape(w)[2] if em is None else em
    call("bcg_bc_extrapolate_o2_2d", arr(w, "w", True), _loc(loc), interf4(interf), int(im), int(jm), int(gh), int(em))


def _pr(p):
    return interf4(p)


def jn_match_2d(wr, prr, gh1r, gh2r, gh3r, gh4r, imr, jmr, wd, prd, gh1d, gh2d, gh3d, gh4d, imd, jmd, tr, em=None):
    em = shape(wr)[2] if em is None else em
    t = np.ascontiguousarray(np.asarray(tr, dtype=np.int32).ravel())
    call("bcg_jn_match_2d", arr(wr, "wr", True), _pr(prr), gh1r, gh2r, gh3r, gh4r, imr, jmr, arr(wd, "wd"), _pr(prd),
         gh1d, gh2d, gh3d, gh4d, imd, jmd, t, int(em))


def jn_match_geom_2d(wr, prr, gh1r, gh2r, gh3r, gh4r, imr, jmr, wd, prd, gh1d, gh2d, gh3d, gh4d, imd, jmd, tr):
    t = np.ascontiguousarray(np.asarray(tr, dtype=np.int32).ravel())
    call("bcg_jn_match_geom_2d", arr(wr, "wr", True), _pr(prr), gh1r, gh2r, gh3r, gh4r, imr, jmr, arr(wd, "wd"),
         _pr(prd), gh1d, gh2d, gh3d, gh4d, imd, jmd, t)
