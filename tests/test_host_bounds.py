"""Bounds of the library's host pre-processing (bcg_computegeom_2d,
bcg_initblfv, bcg_set_bndbl_2d in csrc/host.cpp; computegeom.F90:3-104,
initialisation.f90:2-58, set_bnd.f90:1-24).

Each array is copied into its own mapping between two pages made inaccessible
(PROT_NONE), once flush against the page after it and once flush against the
page before it, so a read or write one element outside any array stops the
child process with SIGSEGV.  The outputs must equal those of the same calls on
ordinary numpy arrays bit for bit.  Runs on the CPU only (these routines need no
GPU).
"""
import os
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent(r"""
    import ctypes, mmap, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    at_end = sys.argv[2] == "end"
    from broadcast_gb300 import _lib, cases

    PAGE = mmap.PAGESIZE
    libc = ctypes.CDLL(None, use_errno=True)
    libc.mprotect.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    keep = []

    def guarded(a):
        body = max(PAGE, -(-a.nbytes // PAGE) * PAGE)
        mm = mmap.mmap(-1, body + 2 * PAGE)
        base = ctypes.addressof(ctypes.c_char.from_buffer(mm))
        for at in (base, base + PAGE + body):
            if libc.mprotect(at, PAGE, 0) != 0:
                raise OSError(ctypes.get_errno(), "mprotect")
        off = PAGE + (body - a.nbytes if at_end else 0)
        v = np.ndarray(a.shape, dtype=a.dtype, buffer=mm, offset=off, order="F")
        v[...] = a
        keep.append(mm)
        return v

    class Ops:
        def __init__(self, guard):
            self.place = guarded if guard else (lambda a: a)

        def _run(self, name, arrays, tail, head=()):
            vs = [self.place(a) for a in arrays]
            _lib.call(name, *head, *[v.ctypes.data for v in vs], *tail)
            for a, v in zip(arrays, vs):
                a[...] = v

        def computegeom(self, x0, y0, nx, ny, xc, yc, vol, volf, im, jm, gh):
            self._run("bcg_computegeom_2d", [x0, y0, nx, ny, xc, yc, vol, volf], (im, jm, gh))

        def initblfv(self, muinf, xc, yc, w, field, im, gh, jm):
            self._run("bcg_initblfv", [xc, yc, w, field], (im, gh, jm), head=(muinf,))

        def set_bndbl(self, w, field, wbd, im, jm, gh):
            self._run("bcg_set_bndbl_2d", [w, field, wbd], (im, jm, gh))

    for im, jm in ((17, 11), (32, 20)):
        a = cases.bl_case(im, jm, seed=1, ops=Ops(True))
        b = cases.bl_case(im, jm, seed=1, ops=Ops(False))
        for k in ("x0", "y0", "nx", "ny", "xc", "yc", "vol", "volf"):
            assert np.array_equal(a["grid"][k], b["grid"][k]), ("bl", im, jm, k)
        for k in ("w", "field", "wbd"):
            assert np.array_equal(a[k], b[k]), ("bl", im, jm, k)
        a = cases.cyl_grid(im + 3, jm, ops=Ops(True))
        b = cases.cyl_grid(im + 3, jm, ops=Ops(False))
        for k in ("x0", "y0", "nx", "ny", "xc", "yc", "vol", "volf"):
            assert np.array_equal(a[k], b[k]), ("cyl", im + 3, jm, k)
    print("ok")
""")


@pytest.mark.parametrize("placement", ["end", "start"])
def test_host_prepro_stays_inside_its_arrays(placement):
    p = subprocess.run([sys.executable, "-c", CHILD, ROOT, placement], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0 and "ok" in p.stdout, (p.returncode, p.stdout[-2000:], p.stderr[-2000:])
