"""Drop-in for the reference's srcfv.f_sch (residual routines).

flux_num_dnc5_2d       : srcfv/rhs/flux_num_dnc5.F90:7-8.
flux_num_dnc5_nowall_2d: srcfv/rhs/flux_num_dnc5_nowall.F90:7 (centred rows everywhere, no wall).
flux_num_dnc{3,7,9}_2d, flux_num_dnc{3,7,9}_nowall_2d: srcfv/rhs/flux_num_dnc{3,7,9}[_nowall].F90:7,
    the schemes of order 3, 7 and 9 (gh >= (order+1)/2; the drivers use gh = (order+1)//2).
"""
from .._f2py import arr, call, dims_from_cell


def flux_num_dnc5_2d(residu, w, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref,
                     s_suth, k2, k4, im=None, jm=None):
    """Residual R(w) of the 5th-order DNC (FE-MUSCL) scheme; writes the
    interior of `residu` in place (not divided by the cell volume)."""
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    residu = arr(residu, "residu", inout=True)
    w, nx, ny, vol, volf = (arr(a, n) for a, n in ((w, "w"), (nx, "nx"), (ny, "ny"), (vol, "vol"), (volf, "volf")))
    call("bcg_flux_num_dnc5_2d", residu, w, None, None, nx, ny, None, None, vol, volf, gh, cp, cv, prandtl, gam, rgaz,
         cs, muref, tref, s_suth, k2, k4, int(im), int(jm))


def flux_num_dnc5_nowall_2d(residu, w, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref,
                            tref, s_suth, k2, k4, im=None, jm=None):
    """The same residual without the wall rows: every row uses the centred fluxes."""
    gh = int(gh)
    if im is None or jm is None:
        im, jm = dims_from_cell(w, gh)
    residu = arr(residu, "residu", inout=True)
    w, nx, ny, vol, volf = (arr(a, n) for a, n in ((w, "w"), (nx, "nx"), (ny, "ny"), (vol, "vol"), (volf, "volf")))
    call("bcg_flux_num_dnc5_nowall_2d", residu, w, None, None, nx, ny, None, None, vol, volf, gh, cp, cv, prandtl,
         gam, rgaz, cs, muref, tref, s_suth, k2, k4, int(im), int(jm))


def _scheme(symbol, doc):
    def residual(residu, w, x0, y0, nx, ny, xc, yc, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref, tref,
                 s_suth, k2, k4, im=None, jm=None):
        gh = int(gh)
        if im is None or jm is None:
            im, jm = dims_from_cell(w, gh)
        residu = arr(residu, "residu", inout=True)
        w, nx, ny, vol, volf = (arr(a, n) for a, n in ((w, "w"), (nx, "nx"), (ny, "ny"), (vol, "vol"), (volf, "volf")))
        call(symbol, residu, w, None, None, nx, ny, None, None, vol, volf, gh, cp, cv, prandtl, gam, rgaz, cs, muref,
             tref, s_suth, k2, k4, int(im), int(jm))
    residual.__name__ = symbol[4:]
    residual.__doc__ = doc
    return residual


flux_num_dnc3_2d = _scheme("bcg_flux_num_dnc3_2d", "Residual of the 3rd-order DNC scheme (srcfv/rhs/flux_num_dnc3.F90:7).")
flux_num_dnc7_2d = _scheme("bcg_flux_num_dnc7_2d", "Residual of the 7th-order DNC scheme (srcfv/rhs/flux_num_dnc7.F90:7).")
flux_num_dnc9_2d = _scheme("bcg_flux_num_dnc9_2d", "Residual of the 9th-order DNC scheme (srcfv/rhs/flux_num_dnc9.F90:7).")
flux_num_dnc3_nowall_2d = _scheme("bcg_flux_num_dnc3_nowall_2d",
                                  "DNC3 without the wall rows (srcfv/rhs/flux_num_dnc3_nowall.F90:7).")
flux_num_dnc7_nowall_2d = _scheme("bcg_flux_num_dnc7_nowall_2d",
                                  "DNC7 without the wall rows (srcfv/rhs/flux_num_dnc7_nowall.F90:7).")
flux_num_dnc9_nowall_2d = _scheme("bcg_flux_num_dnc9_nowall_2d",
                                  "DNC9 without the wall rows (srcfv/rhs/flux_num_dnc9_nowall.F90:7).")
