"""Test infrastructure only: build oracle/_ref/libref.so from the reference's
own Fortran routines (translated to C by oracle/ref_translate.py, compiled by
gcc with -ffp-contract=off).

Runs only where the reference checkout is present:
    python oracle/ref_build.py [reference_root]
The root defaults to $BROADCAST_REFERENCE_ROOT, else /root/reference.
Outputs go to oracle/_ref/ (git-ignored): libref.c, libref.so, signatures.json.
"""
import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
DEFAULT_REF = os.environ.get("BROADCAST_REFERENCE_ROOT", "/root/reference")

# (file relative to the reference root, routines taken from it)
ROUTINES = [
    ("srcfv/prepro/flux_num_dnc5.f90", ["flux_num_dnc5_2d"]),
    ("srcfv/prepro/flux_num_dnc5_nowall.f90", ["flux_num_dnc5_nowall_2d"]),
    ("srcfv/tangent/flux_num_dnc5_nowall_d.f90", ["flux_num_dnc5_nowall_2d_d"]),
    ("srcfv/tangent/flux_num_dnc5_d.f90", ["flux_num_dnc5_2d_d"]),
    ("srcfv/adjoint/flux_num_dnc5_b.f90", ["flux_num_dnc5_2d_b"]),
    ("srcfv/adjoint/flux_num_dnc5_nowall_b.f90", ["flux_num_dnc5_nowall_2d_b"]),
    ("srcfv/prepro/flux_num_dnc3.f90", ["flux_num_dnc3_2d"]),
    ("srcfv/prepro/flux_num_dnc3_nowall.f90", ["flux_num_dnc3_nowall_2d"]),
    ("srcfv/tangent/flux_num_dnc3_d.f90", ["flux_num_dnc3_2d_d"]),
    ("srcfv/tangent/flux_num_dnc3_nowall_d.f90", ["flux_num_dnc3_nowall_2d_d"]),
    ("srcfv/prepro/flux_num_dnc7.f90", ["flux_num_dnc7_2d"]),
    ("srcfv/prepro/flux_num_dnc7_nowall.f90", ["flux_num_dnc7_nowall_2d"]),
    ("srcfv/tangent/flux_num_dnc7_d.f90", ["flux_num_dnc7_2d_d"]),
    ("srcfv/tangent/flux_num_dnc7_nowall_d.f90", ["flux_num_dnc7_nowall_2d_d"]),
    ("srcfv/prepro/flux_num_dnc9.f90", ["flux_num_dnc9_2d"]),
    ("srcfv/prepro/flux_num_dnc9_nowall.f90", ["flux_num_dnc9_nowall_2d"]),
    ("srcfv/tangent/flux_num_dnc9_d.f90", ["flux_num_dnc9_2d_d"]),
    ("srcfv/tangent/flux_num_dnc9_nowall_d.f90", ["flux_num_dnc9_nowall_2d_d"]),
    ("srcfv/prepro/bc_wall_viscous.f90", ["bc_wall_viscous_adia_2d"]),
    ("srcfv/prepro/bc_no_reflexion.f90", ["bc_no_reflexion_2d"]),
    ("srcfv/prepro/bc_supandsubinlet.f90", ["bc_supandsubinlet_2d"]),
    ("srcfv/prepro/bc_extrapolate.f90", ["bc_extrapolate_o2_2d"]),
    ("srcfv/tangent/bc_wall_viscous_d.f90", ["bc_wall_viscous_adia_2d_d"]),
    ("srcfv/tangent/bc_no_reflexion_d.f90", ["bc_no_reflexion_2d_d"]),
    ("srcfv/tangent/bc_supandsubinlet_d.f90", ["bc_supandsubinlet_2d_d"]),
    ("srcfv/tangent/bc_extrapolateo2_d.f90", ["bc_extrapolate_o2_2d_d"]),
    ("srcfv/adjoint/bc_wall_viscous_b.f90", ["bc_wall_viscous_adia_2d_b"]),
    ("srcfv/adjoint/bc_no_reflexion_b.f90", ["bc_no_reflexion_2d_b"]),
    ("srcfv/adjoint/bc_supandsubinlet_b.f90", ["bc_supandsubinlet_2d_b"]),
    ("srcfv/adjoint/bc_extrapolateo2_b.f90", ["bc_extrapolate_o2_2d_b"]),
    ("srcfv/adjoint/jn_match_2d_b.f90", ["jn_match_2d_b"]),
    ("srcfv/prepro/jn_match.f90", ["jn_match_2d"]),
    ("srcfv/prepro/jn_match_geom.f90", ["jn_match_geom_2d"]),
    ("misc/ComputeJacobian.f90", ["testvector", "testvector_partial", "computejacobianfromjv",
                                  "computejacobianfromjv_relaxed", "computejacobianfromjv_relaxed_withjn",
                                  "computejacobianfromjv_withjn", "computejacobianfromjv_relaxed_withjnandcheck",
                                  "computejacobianfromdz"]),
    ("srcfv/norm.F90", ["compute_norml2", "compute_norml2inf", "compute_maxnorm"]),
    # compiled by f2py from the raw sources with their #include fragments
    # (srcfv/compile_dz.py runs fpp with -I srcfv/)
    ("srcfv/dz/coeffs_5p_dz.F90", ["function_5p_dz_d", "coeffs_5p_dz"]),
    ("srcfv/dz/coeffs_5p_dz2.F90", ["function_5p_dz2_d", "coeffs_5p_dz2"]),
    ("srcfv/prepro/computegeom.f90", ["computegeom_2d"]),
    ("srcfv/prepro/impli_matrix_free.f90", ["impli_matrix_free_2d"]),
    ("initialisation.f90", ["initblfv"]),
    ("set_bnd.f90", ["set_bndbl_2d"]),
]


def _resolve_includes(path, inc_root):
    """Expand `#include "x"` lines (paths relative to inc_root), as fpp does."""
    out = []
    for line in open(path, errors="replace"):
        m = re.match(r'\s*#include\s+"([^"]+)"', line)
        out.append(_resolve_includes(os.path.join(inc_root, m.group(1)), inc_root) if m else line)
    return "".join(out)


def _up_to_date():
    so = os.path.join(OUT, "libref.so")
    if not (os.path.exists(so) and os.path.exists(os.path.join(OUT, "signatures.json"))):
        return False
    t = os.path.getmtime(so)
    return all(os.path.getmtime(os.path.join(HERE, f)) < t for f in ("ref_translate.py", "ref_build.py"))


def build(ref_root=DEFAULT_REF, routines=ROUTINES, verbose=False, force=False):
    """Translate and compile; skipped when oracle/_ref is newer than the
    translator and this routine list (the reference sources do not change)."""
    if not force and routines is ROUTINES and _up_to_date():
        return os.path.join(OUT, "libref.so"), []
    sys.path.insert(0, HERE)
    import ref_translate as rt
    if not os.path.isdir(ref_root):
        raise FileNotFoundError("reference checkout not found at %s" % ref_root)
    os.makedirs(OUT, exist_ok=True)
    tr = rt.Translator()
    failures = []
    for rel, names in routines:
        path = os.path.join(ref_root, rel)
        text = _resolve_includes(path, os.path.join(ref_root, "srcfv"))
        before = len(tr.subs)
        try:
            tr.translate_text(text, only=set(names))
        except rt.TranslateError as e:
            failures.append((rel, str(e)))
            del tr.subs[before:]
            continue
        got = {s.name for s in tr.subs[before:]}
        for n in names:
            if n not in got:
                failures.append((rel, "routine %s not found" % n))
    good = []
    for s in tr.subs:
        try:
            code = tr._emit_sub(s)
            good.append((s, code))
        except rt.TranslateError as e:
            failures.append((s.name, str(e)))
    src = rt.PRELUDE + "\n" + "\n\n".join(c for _, c in good) + "\n"
    cfile = os.path.join(OUT, "libref.c")
    open(cfile, "w").write(src)
    sigs = {s.name: [(a, s.vars[a].typ, bool(s.vars[a].dims)) for a in s.args] for s, _ in good}
    json.dump(sigs, open(os.path.join(OUT, "signatures.json"), "w"), indent=1)
    so = os.path.join(OUT, "libref.so")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-w", "-o", so, cfile, "-lm"], check=True)
    if verbose:
        for f in failures:
            print("not translated:", f)
        print("translated:", sorted(sigs))
    return so, failures


if __name__ == "__main__":
    so, fails = build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF, verbose=True, force=True)
    print(so)
