"""Drop-in for the reference's srcfv.f_adj (Tapenade reverse-mode routines).

flux_num_dnc5_2d_b: srcfv/adjoint/flux_num_dnc5_b.f90:15 -- wb = (dR/dw)^T residub
on every padded cell (wb overwritten); the interior of residub is zeroed.
"""
from .._f2py import arr, call, dims_from_cell


def flux_num_dnc5_2d_b(residu, residub, w, wb, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs,
                       muref, tref, s_suth, k2, k4, im=None, jm=None):
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    call("bcg_flux_num_dnc5_2d_b", None, arr(residub, "residub", True), arr(w, "w"), arr(wb, "wb", True), None, None,
         arr(nx, "nx"), arr(ny, "ny"), None, None, arr(vol, "vol"), arr(volf, "volf"), gh, cp, cv, prandtl, gam, rgaz,
         cs, muref, tref, s_suth, k2, k4, int(im), int(jm))
