"""Generate tests/golden/npz_tree_bl_10x8.npz: an NPZ tree file written by the
reference's own writeNPZ, fillNPZ and fillNPZ_3D (BROADCAST_npz.py:247-333).

    python tests/golden/make_npz.py [reference_root]

The reference root defaults to $BROADCAST_REFERENCE_ROOT, else /root/reference.
The three functions are read from the driver's source and executed here (the
driver module itself imports MPI and PETSc at its top, which are absent).
Inputs: the 10 x 8 boundary layer of tests/helpers.bl_case (seed 0, built by
the oracle), a zero residual, the drivers' routine list, the scheme name
"dnc5", and small (IA, JA, Aij) lists; tests/test_npz.py rebuilds the same
inputs to read the file and to compare what this package writes with it.
"""
import ast
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests import helpers as H  # noqa: E402

OUT = os.path.join(HERE, "npz_tree_bl_10x8")
LF = ["bc_supandsubinlet_2d", "bc_extrapolate_o2_2d", "bc_no_reflexion_2d", "bc_wall_viscous_adia_2d",
      "flux_num_dnc5_2d", "f_bnd", "f_sch"]


def inputs():
    """The writer's arguments and the lists filled in afterwards."""
    c = H.bl_case(10, 8)
    g, ph, it = c["grid"], c["phys"], c["interf"]
    args = (g["im"], g["jm"], g["gh"], c["w"], g["x0"], g["y0"], g["vol"], g["volf"], g["nx"], g["ny"], g["xc"],
            g["yc"], c["field"], c["wbd"], np.zeros_like(c["w"]), "dnc5", ph["k2"], ph["k4"], it["Ilo"], it["Ihi"],
            it["Jlo"], it["Jhi"], LF, ph["cp"], ph["cv"], ph["gam"], ph["cs"], ph["tref"], ph["muref"], ph["rgaz"],
            0.5, ph["prandtl"], 1.0e10, 10, 100)
    ia = np.array([0, 1, 5, 7], np.int32)
    ja = np.array([1, 0, 5, 2], np.int32)
    a = np.array([1.5, -2.0, 0.25, 3.0])
    w_end = np.asfortranarray(c["w"] * 1.5)
    r_end = np.asfortranarray(np.full_like(c["w"], 1e-3))
    fill = (w_end, r_end, ia, ja, a, g["gh"])
    fill3 = (ia, ja, 2.0 * a, ja, ia, -a)
    return args, fill, fill3


def reference_functions(root):
    src = open(os.path.join(root, "BROADCAST_npz.py")).read()
    ns = {"_np": np, "print": lambda *a, **k: None}
    for node in ast.parse(src).body:
        if isinstance(node, ast.FunctionDef) and node.name in ("writeNPZ", "fillNPZ", "fillNPZ_3D", "readNPZtree"):
            exec(ast.get_source_segment(src, node), ns)
    return ns


def main(root):
    ref = reference_functions(root)
    args, fill, fill3 = inputs()
    ref["writeNPZ"](OUT, *args, pinf=1.0)
    ref["fillNPZ"](OUT, *fill)
    ref["fillNPZ_3D"](OUT, *fill3)
    t = ref["readNPZtree"](OUT)
    assert len(t) == 36 and np.array_equal(t[3], fill[0])
    print("wrote", OUT + ".npz")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BROADCAST_REFERENCE_ROOT", "/root/reference"))
