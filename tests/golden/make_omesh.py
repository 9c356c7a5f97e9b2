"""Generate tests/golden/omesh_metrics.npz: the O-mesh metrics the reference's
cylinder driver builds, by executing its own statements.

    python tests/golden/make_omesh.py [reference_root]

The reference root defaults to $BROADCAST_REFERENCE_ROOT, else /root/reference.
cylinder.py:478-525 (inside the driver's long setup function) sets the join
ranges, copies the node coordinates into the padded arrays, calls
computegeom_2d, joins xc, yc and vol with jn_match_geom_2d and the face normals
with the state join jn_match_2d over node columns im+2..im+1+gh and
1-gh..0, and forms volf.  Those statements are read from the source and
executed here with the reference's routines translated to C
(oracle/_ref/libref.so, built by oracle/ref_build.py) standing in for the f2py
modules, on the node coordinates of broadcast_gb300.cases.cyl_grid, for an
O-mesh whose im is a multiple of 7 and one whose im is odd (and not a multiple of 7).
"""
import os
import sys
import textwrap
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from broadcast_gb300 import cases  # noqa: E402
from oracle import ref  # noqa: E402
from tests import helpers as H  # noqa: E402

OUT = os.path.join(HERE, "omesh_metrics.npz")
SIZES = ((14, 8), (15, 10))
METRICS = ("nx", "ny", "xc", "yc", "vol", "volf")


def _f2py(name, append_em=False):
    """The translated routine called the way f2py calls it: integer arrays
    converted to int32 Fortran order, the trailing em inferred."""
    def call(*args):
        args = [np.asfortranarray(a, dtype=np.int32) if isinstance(a, np.ndarray) and a.dtype.kind == "i" else a
                for a in args]
        if append_em:
            args.append(args[0].shape[2] if args[0].ndim == 3 else 1)
        ref.call(name, *args)
    return call


def driver_block(root):
    lines = open(os.path.join(root, "cylinder.py")).read().splitlines()
    i0 = next(i for i, l in enumerate(lines) if l.strip().startswith("jmin = 1-gh"))
    i1 = next(i for i in range(i0, len(lines)) if "volf[i,j,1] = 2./(vol[i,j]+vol[i,j-1])" in lines[i])
    return textwrap.dedent("\n".join(lines[i0:i1 + 1]))


def nodes(im, jm):
    """The node coordinates of cases.cyl_grid (interior nodes, (im+1, jm+1))."""
    got = {}

    class Capture(H.OracleOps):
        @staticmethod
        def computegeom(x0, y0, *rest):
            gh = cases.GH
            got["x"] = x0[gh:gh + im + 1, gh:gh + jm + 1].copy()
            got["y"] = y0[gh:gh + im + 1, gh:gh + jm + 1].copy()
            H.OracleOps.computegeom(x0, y0, *rest)

    cases.cyl_grid(im, jm, ops=Capture)
    return got["x"], got["y"]


def main(root):
    if not ref.available():
        raise SystemExit("oracle/_ref is not built: python oracle/ref_build.py")
    block = driver_block(root)
    out = {}
    for im, jm in SIZES:
        gh = cases.GH
        ni, nj = im + 2 * gh, jm + 2 * gh
        z = lambda *s: np.zeros(s, order="F")
        x, y = nodes(im, jm)
        ns = {"_np": np, "im": im, "jm": jm, "gh": gh, "x": x, "y": y,
              "x0": z(ni + 1, nj + 1), "y0": z(ni + 1, nj + 1), "nx": z(ni + 1, nj + 1, 2), "ny": z(ni + 1, nj + 1, 2),
              "xc": z(ni, nj), "yc": z(ni, nj), "vol": z(ni, nj), "volf": z(ni, nj, 2),
              "f_geom": types.SimpleNamespace(computegeom_2d=_f2py("computegeom_2d")),
              "f_bnd": types.SimpleNamespace(jn_match_geom_2d=_f2py("jn_match_geom_2d")),
              "fjn": _f2py("jn_match_2d", append_em=True)}
        exec(block, ns)
        for k in METRICS:
            out["%s_%dx%d" % (k, im, jm)] = ns[k]
    np.savez(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BROADCAST_REFERENCE_ROOT", "/root/reference"))
