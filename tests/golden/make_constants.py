"""Generate tests/golden/constants.json: the nondimensional constants the
reference's drivers compute, by executing the reference's own statements.

    python tests/golden/make_constants.py [reference_root]

The reference root defaults to $BROADCAST_REFERENCE_ROOT, else /root/reference.
Both drivers turn a card's dimensional constants into the constants the
residual routines take inside one long function, so the statements from
"# get physical constants" through the state_adim assignment are read from
the driver's source (BROADCAST_npz.py:555-669 for the boundary layer with
Lref = mu_inf / (rho_inf u_inf); cylinder.py:298-400 for the cylinder with
Lref = D) and executed with the driver's own __comp_Sutherland and
__compute_tot_energy_inf, on the physical constants of card_bl2d_fv_npz.py and
card_cyl2d.py at the Mach and Reynolds numbers of this project's workloads.
Printing is switched off; the grid quantities the block only prints (dx, dt)
get placeholder values.
"""
import ast
import json
import os
import sys
import textwrap

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "constants.json")
KEYS = ("gam", "cp", "cv", "rgaz", "prandtl", "cs", "muref", "tref", "muinf", "einf", "pinf")


def card_dphys(path):
    """The card's module-level dphys['key'] = literal assignments."""
    d = {}
    for node in ast.parse(open(path).read()).body:
        if isinstance(node, ast.Assign) and len(node.targets) == 1:
            t = node.targets[0]
            if (isinstance(t, ast.Subscript) and isinstance(t.value, ast.Name) and t.value.id == "dphys"
                    and isinstance(t.slice, ast.Constant)):
                d[t.slice.value] = ast.literal_eval(node.value)
    return d


def driver_block(path):
    """(helper function sources, the constants block) of a driver file."""
    src = open(path).read()
    helpers = [ast.get_source_segment(src, n) for n in ast.parse(src).body
               if isinstance(n, ast.FunctionDef) and n.name in ("__comp_Sutherland", "__compute_tot_energy_inf")]
    assert len(helpers) == 2, path
    lines = src.splitlines()
    i0 = next(i for i, l in enumerate(lines) if "# get physical constants" in l)
    i1 = next(i for i in range(i0, len(lines)) if "state_adim[4]" in lines[i])
    return "\n".join(helpers), textwrap.dedent("\n".join(lines[i0:i1 + 1]))


def run(path, dphys, **grid):
    helpers, block = driver_block(path)
    ns = {"_np": np, "print": lambda *a, **k: None, "dphys": dict(dphys), "cfl": 1.0, "sch": "dnc", "order": 5}
    ns.update(grid)
    exec(helpers, ns)
    exec(block, ns)
    out = {k: float(ns[k]) for k in KEYS}
    out["state"] = [float(v) for v in ns["state_adim"]]
    return out


def main(root):
    bl_card = card_dphys(os.path.join(root, "card_bl2d_fv_npz.py"))
    cyl_card = card_dphys(os.path.join(root, "card_cyl2d.py"))
    table = {"bl": [], "cyl": []}
    for mach in (0.3, 0.5, 0.8):
        d = dict(bl_card, Mach=mach)
        c = run(os.path.join(root, "BROADCAST_npz.py"), d, L=1.0, im=11, y=np.array([0.0, 1.0]))
        table["bl"].append({"mach": mach, "runit": d["Runit"], "constants": c})
    for mach, re in ((0.1, 47.0), (0.05, 40.0), (0.3, 200.0)):
        # cylinder.py:358: Re_D = Runit * 2 rint with rint = 0.5 (card_cyl2d.py:46)
        d = dict(cyl_card, Mach=mach, Runit=re)
        c = run(os.path.join(root, "cylinder.py"), d, x=np.array([[0.0, 1.0]]), rint=0.5)
        table["cyl"].append({"mach": mach, "reynolds": re, "constants": c})
    json.dump(table, open(OUT, "w"), indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BROADCAST_REFERENCE_ROOT", "/root/reference"))
