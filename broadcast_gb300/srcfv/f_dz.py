"""Drop-in for the reference's srcfv.f_dz (spanwise operators, 5-point gradients).

coeffs_5p_dz : srcfv/dz/coeffs_5p_dz.F90:10  -- dz_out = Dz . wd  (coefficient of i*beta)
coeffs_5p_dz2: srcfv/dz/coeffs_5p_dz2.F90:10 -- dz2_out = Dzz . wd (coefficient of -beta^2)
The interior of the output array is written, its ghosts are left as they are
(intent(inout) in the reference).  Called by BROADCAST_npz.py:1238-1239.
"""
from .._f2py import arr, call, dims_from_cell


def _span(name, out, w, wd, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref,
          s_suth, im, jm):
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    call(name, arr(out, "dz_out", True), arr(w, "w"), arr(wd, "wd"), None, None, arr(nx, "nx"), arr(ny, "ny"), None,
         None, arr(vol, "vol"), None, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref, s_suth, int(im), int(jm))


def coeffs_5p_dz(dz_out, w, wd, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref,
                 s_suth, im=None, jm=None):
    _span("bcg_coeffs_5p_dz", dz_out, w, wd, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs,
          muref, tref, s_suth, im, jm)


def coeffs_5p_dz2(dz2_out, w, wd, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref,
                  s_suth, im=None, jm=None):
    _span("bcg_coeffs_5p_dz2", dz2_out, w, wd, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs,
          muref, tref, s_suth, im, jm)
