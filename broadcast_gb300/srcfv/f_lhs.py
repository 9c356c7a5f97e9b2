"""Drop-in for the reference's srcfv.f_lhs (implicit left-hand-side routines).

impli_matrix_free_2d: srcfv/lhs/impli_matrix_free.F90:7, called by the 'impli'
time marching as fimpli(dw, nx, ny, w, res, vol, volf, dtcoef, cfl, gam, rgaz,
prandtl, lmax, gh, cv, cs, muref, tref, cs, im, jm) (BROADCAST_npz.py:941).
"""
from .._f2py import arr, call, dims_from_cell


def impli_matrix_free_2d(dwi, nx, ny, w, dw, vol, volf, dtcoef, cfl, gam, rgaz, prandtl, lmax, gh, cv, cs, muref, tref,
                         s_suth, im=None, jm=None, em=None):
    """lmax symmetric Gauss-Seidel sweeps of the matrix-free implicit operator on
    the right-hand side dw; dwi (in place) receives the increment, ghosts zero."""
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    em = 5 if em is None else int(em)
    call("bcg_impli_matrix_free_2d", arr(dwi, "dwi", True), arr(nx, "nx"), arr(ny, "ny"), arr(w, "w"), arr(dw, "dw"),
         arr(vol, "vol"), arr(volf, "volf"), dtcoef, cfl, gam, rgaz, prandtl, int(lmax), gh, cv, cs, muref, tref, s_suth,
         int(im), int(jm), em)
