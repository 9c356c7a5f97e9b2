"""Loading of the golden fixtures (tests/golden/*.npz, made from the
reference's own routines by tests/golden/make_golden.py)."""
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PHYS = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")
CASES = ["bl_14x10", "cyl_14x8", "bl_23x17"]
# the DNC schemes of order 3, 7 and 9 (gh = (order+1)//2)
SCHEME_CASES = ["dnc%d_%s_12x11" % (o, k) for o in (3, 7, 9) for k in ("bl", "cyl")]
# impli_matrix_free_2d on the residual of a small case, lmax = 1, 2, 10
IMPLI_CASES = ["impli_bl_16x10", "impli_cyl_14x8"]
# flux_num_dnc5_nowall_2d_b on one cotangent (k2 = 1.01 on the boundary layer, 0 on the cylinder)
NOWALL_ADJ_CASES = ["adj_nowall_bl_16x12", "adj_nowall_cyl_16x12"]


def load(name):
    z = np.load(os.path.join(HERE, name + ".npz"))
    d = {k: z[k] for k in z.files}
    for k, v in list(d.items()):
        if isinstance(v, np.ndarray) and v.ndim >= 2:
            if v.ndim == 4:  # stacks of padded states
                d[k] = np.stack([np.asfortranarray(x) for x in v])
            else:
                d[k] = np.asfortranarray(v)
        elif isinstance(v, np.ndarray) and v.ndim == 0:
            d[k] = v.item()
    return d


def as_case(d):
    """Case dictionary in the layout of broadcast_gb300.cases."""
    from broadcast_gb300 import cases
    im, jm, gh = int(d["im"]), int(d["jm"]), int(d["gh"])
    grid = {k: d[k] for k in ("x0", "y0", "nx", "ny", "xc", "yc", "vol", "volf")}
    grid.update(im=im, jm=jm, gh=gh)
    phys = {k: float(d["phys_" + k]) for k in PHYS}
    kind = str(d["kind"])
    c = dict(kind=kind, grid=grid, phys=phys, w=d["w"].copy(order="F"), wbd=d["wbd"])
    if kind == "bl":
        c["field"] = d["field"]
        c["interf"] = cases.bl_interfaces(im, jm, gh)
    else:
        c["interf"] = cases.cyl_interfaces(im, jm, gh)
    return c
