"""Drop-in for the reference's f_init module (initialisation.f90, set_bnd.f90)."""
from ._f2py import arr, call, shape


def set_bndbl_2d(w, field, wbd, im, jm=None, gh=None):
    """set_bnd.f90:1-24"""
    field = arr(field, "field", True)
    jm = shape(field)[0] if jm is None else jm
    gh = shape(field)[1] if gh is None else gh
    call("bcg_set_bndbl_2d", arr(w, "w"), field, arr(wbd, "wbd", True), int(im), int(jm), int(gh))


def initblfv(muinf, xc, yc, w, field, im, gh=None, jm=None):
    """initialisation.f90:2-58"""
    field = arr(field, "field", True)
    jm = shape(field)[0] if jm is None else jm
    gh = shape(field)[1] if gh is None else gh
    call("bcg_initblfv", muinf, arr(xc, "xc"), arr(yc, "yc"), arr(w, "w", True), field, int(im), int(gh), int(jm))
