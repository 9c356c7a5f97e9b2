"""Drop-in for the reference's srcfv.f_norm (srcfv/norm.F90)."""
import numpy as np

from .._f2py import arr, call, dims_from_cell


def _dims(rhs, im, jm, gh):
    if gh is None:
        gh = 3
    if im is None or jm is None:
        im, jm = dims_from_cell(rhs, gh)
    return int(im), int(jm), int(gh)


def compute_norml2(rhs, im=None, jm=None, gh=None):
    """norm.F90:2-32 -> (norm, nmoy)"""
    im, jm, gh = _dims(rhs, im, jm, gh)
    a, b = np.zeros(5), np.zeros(5)
    call("bcg_compute_norml2", a, b, arr(rhs, "rhs"), im, jm, gh)
    return a, b


def compute_norml2inf(rhs, im=None, jm=None, gh=None):
    """norm.F90:34-77 -> (norm, ninf); ninf = (sum r**10)**0.1"""
    im, jm, gh = _dims(rhs, im, jm, gh)
    a, b = np.zeros(5), np.zeros(5)
    call("bcg_compute_norml2inf", a, b, arr(rhs, "rhs"), im, jm, gh)
    return a, b


def compute_maxnorm(rhs, im=None, jm=None, gh=None):
    """norm.F90:79-127 -> (norm, imax, jmax)"""
    im, jm, gh = _dims(rhs, im, jm, gh)
    a = np.zeros(5)
    i, j = np.zeros(5, np.int32), np.zeros(5, np.int32)
    call("bcg_compute_maxnorm", a, i, j, arr(rhs, "rhs"), im, jm, gh)
    return a, i, j
