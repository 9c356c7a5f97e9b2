"""Drop-in for the reference's srcfv.f_geom (geom/computegeom.F90:3)."""
from .._f2py import arr, call


def computegeom_2d(x0, y0, nx, ny, xc, yc, vol, volf, im, jm, gh):
    call("bcg_computegeom_2d", *(arr(a, n, True) for a, n in ((x0, "x0"), (y0, "y0"), (nx, "nx"), (ny, "ny"),
                                                               (xc, "xc"), (yc, "yc"), (vol, "vol"), (volf, "volf"))),
         int(im), int(jm), int(gh))
