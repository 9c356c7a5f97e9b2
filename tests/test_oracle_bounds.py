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

import pytest

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


# Every oracle entry point with its arrays in guarded memory: oracle._p (where
# the wrappers turn arrays into pointers) is replaced by a copy into a mapping
# between two PROT_NONE pages, flush against one of them, and the copies are
# written back after each call.  The outputs must equal an unguarded run bit for
# bit.
SWEEP = textwrap.dedent(r"""
    import ctypes, mmap, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    at_end = sys.argv[2] == "end"
    from oracle import oracle as O
    from tests import helpers as H

    PAGE = mmap.PAGESIZE
    libc = ctypes.CDLL(None, use_errno=True)
    libc.mprotect.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    keep, pending = [], {}

    def guarded(a):
        assert a.flags.f_contiguous or a.flags.c_contiguous, "strided array passed as a pointer"
        body = max(PAGE, -(-a.nbytes // PAGE) * PAGE)
        mm = mmap.mmap(-1, body + 2 * PAGE)
        base = ctypes.addressof(ctypes.c_char.from_buffer(mm))
        for at in (base, base + PAGE + body):
            if libc.mprotect(at, PAGE, 0) != 0:
                raise OSError(ctypes.get_errno(), "mprotect")
        off = PAGE + (body - a.nbytes if at_end else 0)
        v = np.ndarray(a.shape, dtype=a.dtype, buffer=mm, offset=off, order="F" if a.flags.f_contiguous else "C")
        v[...] = a
        keep.append(mm)
        return v

    def gp(a):
        if a is None:
            return None
        key = a.ctypes.data
        if key not in pending:
            pending[key] = (a, guarded(a))
        return pending[key][1].ctypes.data

    class Proxy:
        def __init__(self, real):
            self.real = real

        def __getattr__(self, name):
            fn = getattr(self.real, name)

            def call(*args):
                try:
                    return fn(*args)
                finally:
                    for src, v in pending.values():
                        src[...] = v
                    pending.clear()
            return call

    def run():
        out = []
        rng = np.random.default_rng(11)
        bl, cy, bl5 = H.bl_case(17, 11, seed=1), H.cyl_case(15, 12, seed=1), H.bl_case(16, 13, seed=2, gh=5)
        for c in (bl, cy):
            g, ph = c["grid"], c["phys"]
            im, jm, gh = g["im"], g["jm"], g["gh"]
            out += [g[k] for k in ("nx", "ny", "xc", "yc", "vol", "volf")]
            w = c["w"].copy(order="F")
            H.oracle_bcs(c, w)
            wd = np.asfortranarray(rng.standard_normal(w.shape))
            wt = c["w"].copy(order="F")
            H.oracle_bcs(c, wt, wd)
            out += [w, wt, wd]
            res = O.residual(g, ph, w)
            out += [res, O.residual(g, ph, w, nowall=True)]
            for nd in (1, 3, 5):
                stack = np.stack([np.asfortranarray(rng.standard_normal(w.shape)) for _ in range(nd)])
                for omp in (False, True):
                    out += list(O.jvp(g, ph, w, stack if nd > 1 else stack[0], openmp=omp))
                out += list(O.jvp(g, ph, w, stack, nowall=True))
                out += [O.dz(g, ph, w, stack), O.dzz(g, ph, w, stack)]
            rb = np.asfortranarray(rng.standard_normal(w.shape))
            out += [O.vjp(g, ph, w, rb), O.vjp(g, ph, w, rb, nowall=True)]
            out += [O.impli_matrix_free(g, ph, w, res, 1.0, 5.0, 2)]
            out += [O.opcount(g, ph, w)[0]]
            out += list(O.norml2(res, im, jm, gh)) + list(O.norml2inf(res, im, jm, gh)) + list(O.maxnorm(res, im, jm, gh))
            it = c["interf"]
            kinds = (("inlet", "Ilo"), ("noref", "Jhi"), ("extrap", "Ihi"), ("wall", "Jlo")) if c["kind"] == "bl" \
                else (("noref", "Jhi"), ("wall", "Jlo"))
            for kind, loc in kinds:
                wb = np.asfortranarray(rng.standard_normal(w.shape))
                aux = {"inlet": c.get("field"), "noref": c["wbd"]}.get(kind)
                out += [O.bc_adjoint(kind, w.copy(order="F"), wb, loc, it[loc], gh, im, jm, gam=ph["gam"], aux=aux,
                                     nx=g["nx"], ny=g["ny"])]
            seeds = [(0, 0, 0), (2, 3, 5), (4, 6, 6)]
            nb = im * jm * 49 * 25
            cd = np.asfortranarray(rng.uniform(1.0, 2.0, (im, jm)))
            for mode in range(5):
                jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
                for (m, l, k) in seeds:
                    t = O.testvector(m, l, k, gh, im, jm)
                    _, rd = O.jvp(g, ph, w, t)
                    O.computejacobian(mode, jac, ia, ja, rd, m, l, k, gh, im, jm, cd if mode in (1, 2) else None)
                    out += [t] + list(O.computejacobian_band(mode, rd, m, l, k, gh, im, jm, cd if mode in (1, 2) else None))
                out += [jac, ia, ja]
            jac, ia, ja = np.zeros(2 * nb), np.zeros(2 * nb, np.int32), np.zeros(2 * nb, np.int32)
            for n in (0, 1):
                for (m, l, k) in seeds:
                    t = O.testvector_partial(m, l, k, gh, im, jm, 2, im - 2, 0, jm - 1)
                    _, rd = O.jvp(g, ph, w, t)
                    O.computejacobian_withjnandcheck(jac, ia, ja, rd, m, l, k, gh, im, jm, cd, 2e-16, n)
                    out += [t]
            out += [jac, ia, ja]
        g, ph, w = bl5["grid"], bl5["phys"], bl5["w"]
        wd = np.asfortranarray(rng.standard_normal(w.shape))
        for order in (3, 5, 7, 9):
            for nowall in (False, True):
                out += [O.residual(g, ph, w, order=order, nowall=nowall)]
                out += list(O.jvp(g, ph, w, np.stack([wd, 2.0 * wd]), order=order, nowall=nowall))
        return out

    plain = run()
    O.lib(False), O.lib(True)
    for key in list(O._libs):
        O._libs[key] = Proxy(O._libs[key])
    O._p = gp
    got = run()
    assert len(got) == len(plain)
    for q, (a, b) in enumerate(zip(got, plain)):
        a, b = np.asarray(a), np.asarray(b)
        assert a.shape == b.shape and np.array_equal(a, b, equal_nan=a.dtype.kind == "f"), q
    print("ok", len(got))
""")


@pytest.mark.parametrize("placement", ["end", "start"])
def test_oracle_entry_points_stay_inside_their_arrays(placement):
    p = subprocess.run([sys.executable, "-c", SWEEP, ROOT, placement], capture_output=True, text=True, timeout=600)
    assert p.returncode == 0 and "ok" in p.stdout, (p.returncode, p.stdout[-2000:], p.stderr[-3000:])
