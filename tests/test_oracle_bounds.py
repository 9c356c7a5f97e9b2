"""The oracle's multi-direction tangent reads only the directions it is given.

orc_flux_num_dnc5_2d_d runs groups of up to 8 directions through one dual
number type (1, 2, 4 or 8 slots); a group of 5 directions uses the 8-slot type.
The tangent stack is placed so that it ends exactly at a page made
inaccessible (PROT_NONE): a read of any plane past the 5 given would stop the
child process with SIGSEGV.  The child also checks each direction against a
one-direction call.  Runs on the CPU only.
"""
import os
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent(r"""
    import ctypes, mmap, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    from oracle import oracle as O
    from tests import helpers as H

    c = H.bl_case(18, 14, seed=2)
    g, ph, w = c["grid"], c["phys"], c["w"]
    n, nd = w.size, 5
    rng = np.random.default_rng(7)
    wds = [np.asfortranarray(rng.standard_normal(w.shape)) for _ in range(nd)]

    page = mmap.PAGESIZE
    nbytes = nd * n * 8
    body = -(-nbytes // page) * page
    mm = mmap.mmap(-1, body + page)
    base = ctypes.addressof(ctypes.c_char.from_buffer(mm))
    off = body - nbytes
    libc = ctypes.CDLL(None, use_errno=True)
    libc.mprotect.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    if libc.mprotect(base + body, page, 0) != 0:
        raise OSError(ctypes.get_errno(), "mprotect")
    stack = np.frombuffer(mm, dtype=np.float64, count=nd * n, offset=off)
    for k in range(nd):
        stack[k * n:(k + 1) * n] = np.ravel(wds[k], order="F")

    res = np.zeros_like(w, order="F")
    out = np.zeros(nd * n)
    phys = [ph[k] for k in ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")]
    rc = O.lib().orc_flux_num_dnc5_2d_d(res.ctypes.data, out.ctypes.data, w.ctypes.data, base + off, nd,
                                        g["nx"].ctypes.data, g["ny"].ctypes.data, g["vol"].ctypes.data,
                                        g["volf"].ctypes.data, g["gh"], *phys, g["im"], g["jm"])
    assert rc == 0
    for k in range(nd):
        _, rd1 = O.jvp(g, ph, w, wds[k])
        got = np.reshape(out[k * n:(k + 1) * n], w.shape, order="F")
        scale = np.abs(rd1).max()
        assert np.abs(got - rd1).max() <= 1e-14 * scale, k
    print("ok")
""")


def test_jvp_group_reads_only_its_directions():
    p = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0 and "ok" in p.stdout, (p.returncode, p.stdout[-2000:], p.stderr[-2000:])
