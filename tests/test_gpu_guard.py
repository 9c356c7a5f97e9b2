"""Bounds evidence for the entry points' device kernels: every array is a view
into a larger device buffer whose margins (as long as the array itself, on
both sides) hold a NaN bit pattern.  A read past an input's ends would carry
NaN into the outputs; a write past an output's ends would change a margin.
Each call must leave every margin bit-unchanged, produce finite outputs equal
bit for bit to the same call on ordinary arrays, and leave the ghost cells of
interior-only outputs as the caller set them.  Covered: residual + multi-
direction JVP, VJP, the boundary fills of both drivers, the uneven batch
(with its tile tables), the all-seed Jacobian CSR with its capacity exactly
the entry count, the spanwise operators, and the Krylov solve."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu

NAN_BITS = 0x7FF8DEADBEEF0001
KEYS = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")


class Guarded:
    """A device copy of a host array (or a zero / constant array of a shape
    and dtype) in the middle of a NaN-filled buffer; .f is the array view
    with Fortran strides, .flat the 1-D view."""

    def __init__(self, a=None, shape=None, dtype=np.float64, fill=0.0):
        import torch
        if a is not None:
            a = np.asarray(a)
            shape, dtype = a.shape, a.dtype
        n = int(np.prod(shape)) if len(shape) else 1
        tdt = {np.dtype(np.float64): torch.float64, np.dtype(np.int32): torch.int32}[np.dtype(dtype)]
        self.m = max(n, 1024)
        if tdt == torch.float64:
            self.buf = torch.empty(n + 2 * self.m, dtype=torch.int64, device="cuda")
            self.buf.fill_(NAN_BITS)
            self.buf = self.buf.view(torch.float64)
        else:
            self.buf = torch.full((n + 2 * self.m,), -123456789, dtype=torch.int32, device="cuda")
        self.n, self.shape, self.tdt = n, tuple(shape), tdt
        self.flat = self.buf[self.m:self.m + n]
        if a is not None:
            self.flat.copy_(torch.from_numpy(np.ascontiguousarray(np.ravel(a, order="F"))).to("cuda"))
        else:
            self.flat.fill_(fill)
        rev = tuple(reversed(self.shape))
        self.f = self.flat.view(rev).permute(*reversed(range(len(rev)))) if len(rev) > 1 else self.flat

    def margins_intact(self):
        import torch
        raw = self.buf.view(torch.int64) if self.tdt == torch.float64 else self.buf
        pat = NAN_BITS if self.tdt == torch.float64 else -123456789
        return bool((raw[:self.m] == pat).all()) and bool((raw[self.m + self.n:] == pat).all())

    def host(self):
        return np.reshape(self.flat.cpu().numpy(), self.shape, order="F")


def _check(arrays):
    import torch
    torch.cuda.synchronize()
    for name, g in arrays.items():
        assert g.margins_intact(), "margin of %s changed" % name


def _plain(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.ravel(np.asarray(a), order="F"))).to("cuda")


def _bl():
    c = H.bl_case(41, 29, seed=5)
    H.oracle_bcs(c, c["w"])
    return c


def test_residual_jvp_and_vjp():
    from broadcast_gb300 import _lib
    c = _bl()
    g, ph = c["grid"], c["phys"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    phys = [float(ph[k]) for k in KEYS]
    rng = np.random.default_rng(0)
    K = 3
    wd = np.stack([np.asfortranarray(rng.standard_normal(c["w"].shape)) for _ in range(K)])
    wd_f = np.concatenate([np.ravel(x, order="F") for x in wd])
    G = {k: Guarded(g[k]) for k in ("nx", "ny", "vol", "volf")}
    G["w"] = Guarded(c["w"])
    G["wd"] = Guarded(wd_f)
    G["res"] = Guarded(shape=c["w"].shape, fill=7.0)
    G["resd"] = Guarded(shape=(wd_f.size,), fill=-3.0)
    _lib.call("bcg_flux_num_dnc5_2d_dn", G["res"].flat, G["resd"].flat, G["w"].flat, G["wd"].flat, K, None, None,
              G["nx"].flat, G["ny"].flat, None, None, G["vol"].flat, G["volf"].flat, gh, *phys, im, jm)
    _check(G)
    P = {k: _plain(g[k]) for k in ("nx", "ny", "vol", "volf")}
    res, resd = _plain(np.full(c["w"].shape, 7.0)), _plain(np.full(wd_f.size, -3.0))
    _lib.call("bcg_flux_num_dnc5_2d_dn", res, resd, _plain(c["w"]), _plain(wd_f), K, None, None, P["nx"], P["ny"],
              None, None, P["vol"], P["volf"], gh, *phys, im, jm)
    r_g, rd_g = G["res"].host(), G["resd"].flat.cpu().numpy()
    assert np.isfinite(r_g).all() and np.isfinite(rd_g).all()
    assert np.array_equal(r_g, np.reshape(res.cpu().numpy(), c["w"].shape, order="F"))
    assert np.array_equal(rd_g, resd.cpu().numpy())
    ghost = np.ones(c["w"].shape, bool)
    ghost[gh:-gh, gh:-gh] = False
    assert (r_g[ghost] == 7.0).all()
    # VJP: wb += (dR/dw)^T rb over the padded cells, rb consumed
    rb = np.zeros_like(c["w"])
    rb[gh:-gh, gh:-gh] = rng.standard_normal((im, jm, 5))
    V = {"rb": Guarded(rb), "wb": Guarded(shape=c["w"].shape, fill=0.0), "w": Guarded(c["w"])}
    V.update({k: Guarded(g[k]) for k in ("nx", "ny", "vol", "volf")})
    _lib.call("bcg_flux_num_dnc5_2d_b", None, V["rb"].flat, V["w"].flat, V["wb"].flat, None, None, V["nx"].flat,
              V["ny"].flat, None, None, V["vol"].flat, V["volf"].flat, gh, *phys, im, jm)
    _check(V)
    wb = _plain(np.zeros(c["w"].shape))
    _lib.call("bcg_flux_num_dnc5_2d_b", None, _plain(rb), _plain(c["w"]), wb, None, None, P["nx"], P["ny"], None,
              None, P["vol"], P["volf"], gh, *phys, im, jm)
    assert np.isfinite(V["wb"].host()).all()
    assert np.array_equal(V["wb"].flat.cpu().numpy(), wb.cpu().numpy())


def test_boundary_fills_bl_and_cylinder():
    from broadcast_gb300.srcfv import f_bnd, f_lin
    for c in (H.bl_case(37, 23, seed=2), H.cyl_case(29, 17, seed=3)):
        g, ph, it = c["grid"], c["phys"], c["interf"]
        im, jm, gh = g["im"], g["jm"], g["gh"]
        wd = np.asfortranarray(np.random.default_rng(1).standard_normal(c["w"].shape))
        G = {"w": Guarded(c["w"]), "wd": Guarded(wd), "nx": Guarded(g["nx"]), "ny": Guarded(g["ny"]),
             "wbd": Guarded(c["wbd"])}
        if c["kind"] == "bl":
            G["field"] = Guarded(c["field"])
            f_lin.bc_supandsubinlet_2d_d(G["w"].f, G["wd"].f, "Ilo", it["Ilo"], G["field"].f, G["nx"].f, G["ny"].f,
                                         ph["gam"], im, jm)
            f_lin.bc_no_reflexion_2d_d(G["w"].f, G["wd"].f, G["wbd"].f, "Jhi", it["Jhi"], G["nx"].f, G["ny"].f,
                                       ph["gam"], gh, im, jm)
            f_lin.bc_extrapolate_o2_2d_d(G["w"].f, G["wd"].f, "Ihi", it["Ihi"], im, jm, gh)
            f_lin.bc_wall_viscous_adia_2d_d(G["w"].f, G["wd"].f, "Jlo", ph["gam"], it["Jlo"], gh, im, jm)
        else:
            f_lin.bc_no_reflexion_2d_d(G["w"].f, G["wd"].f, G["wbd"].f, "Jhi", it["Jhi"], G["nx"].f, G["ny"].f,
                                       ph["gam"], gh, im, jm)
            f_lin.bc_wall_viscous_adia_2d_d(G["w"].f, G["wd"].f, "Jlo", ph["gam"], it["Jlo"], gh, im, jm)
            for _ in range(2):
                for a in (G["wd"].f, G["w"].f):
                    f_bnd.jn_match_2d(a, it["prr1"], gh, gh, gh, gh, im, jm, a, it["prd2"], gh, gh, gh, gh, im, jm,
                                      it["tr"])
                    f_bnd.jn_match_2d(a, it["prr2"], gh, gh, gh, gh, im, jm, a, it["prd1"], gh, gh, gh, gh, im, jm,
                                      it["tr"])
        _check(G)
        w_ref, wd_ref = c["w"].copy(order="F"), wd.copy(order="F")
        H.lib_bcs(c, w_ref, wd_ref)
        assert np.isfinite(G["w"].host()).all() and np.isfinite(G["wd"].host()).all()
        assert np.array_equal(G["w"].host(), w_ref) and np.array_equal(G["wd"].host(), wd_ref)


def test_uneven_batch_tile_tables():
    import torch
    from broadcast_gb300 import _lib
    from broadcast_gb300.batch import PHYS_KEYS, CANDIDATES, GridBatch
    from broadcast_gb300.operator import to_device, to_host
    rng = np.random.default_rng(21)
    cases, wds = [], []
    for k in range(5):
        im, jm = int(rng.integers(20, 70)), int(rng.integers(10, 35))
        c = H.bl_case(im, jm, mach=float(rng.uniform(0.3, 0.8)), seed=k)
        H.oracle_bcs(c, c["w"])
        wd = np.zeros_like(c["w"])
        wd[3:-3, 3:-3] = rng.standard_normal((im, jm, 5))
        cases.append(c)
        wds.append(wd)
    n = len(cases)
    ims = np.array([c["grid"]["im"] for c in cases], np.int32)
    jms = np.array([c["grid"]["jm"] for c in cases], np.int32)
    ph = np.ascontiguousarray([[float(c["phys"][k]) for k in PHYS_KEYS] for c in cases])
    h = np.zeros(1, np.int64)
    _lib.call("bcg_set_stream", torch.cuda.current_stream().cuda_stream)
    _lib.call("bcg_batch_create", n, ims, jms, ph, 1, h)
    plan = int(h[0])
    G = []
    for c, wd in zip(cases, wds):
        g = c["grid"]
        G.append({"w": Guarded(c["w"]), "wd": Guarded(wd), "nx": Guarded(g["nx"]), "ny": Guarded(g["ny"]),
                  "vol": Guarded(g["vol"]), "volf": Guarded(g["volf"]),
                  "res": Guarded(shape=c["w"].shape, fill=5.0), "resd": Guarded(shape=c["w"].shape, fill=6.0)})
    tab = lambda k: np.asarray([x[k].flat.data_ptr() for x in G], dtype=np.uint64)
    _lib.call("bcg_batch_set_arrays", plan, tab("w"), tab("wd"), tab("nx"), tab("ny"), tab("vol"), tab("volf"),
              tab("res"), tab("resd"))
    ref = GridBatch([c["grid"] for c in cases], [c["phys"] for c in cases], ndir=1)
    ref.set_states([to_device(c["w"]) for c in cases], [to_device(wd) for wd in wds])
    try:
        for cand in CANDIDATES[::3] + [CANDIDATES[-1]]:
            _lib.call("bcg_batch_configure", plan, *cand)
            _lib.call("bcg_batch_run", plan, 1)
            ref.configure(*cand)
            ref.run(use_graph=False)
            for x in G:
                _check(x)
            for gi, x in enumerate(G):
                r = x["res"].host()
                assert np.isfinite(r).all()
                assert np.array_equal(r[3:-3, 3:-3], to_host(ref.res[gi])[3:-3, 3:-3]), cand
                assert np.array_equal(x["resd"].host()[3:-3, 3:-3], to_host(ref.resd[gi])[3:-3, 3:-3]), cand
                ghost = np.ones(r.shape, bool)
                ghost[3:-3, 3:-3] = False
                assert (r[ghost] == 5.0).all()
    finally:
        _lib.call("bcg_batch_destroy", plan)


def test_jacobian_csr_capacity_exactly_nnz_and_spanwise():
    import torch
    from broadcast_gb300 import _lib
    from broadcast_gb300._f2py import interf4
    c = H.bl_case(23, 16, seed=1)
    H.oracle_bcs(c, c["w"])
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    nrow = 5 * im * jm
    coef = np.asfortranarray(np.random.default_rng(3).uniform(0.5, 2.0, (im, jm)))

    def run(ins, indptr, indices, data, cap):
        nnz = np.zeros(1, np.int64)
        _lib.call("bcg_jacobian_dnc5_bl_csr", ins["w"], ins["nx"], ins["ny"], ins["vol"], ins["volf"], gh,
                  *[float(ph[k]) for k in KEYS], im, jm, interf4(it["Ilo"]), interf4(it["Jhi"]), interf4(it["Ihi"]),
                  interf4(it["Jlo"]), ins["field"], c["field"].shape[0], ins["wbd"], c["wbd"].shape[0], ins["coef"],
                  2e-16, 1, indptr, indices, data, cap, nnz)
        torch.cuda.synchronize()
        return int(nnz[0])

    plain = {k: _plain(v) for k, v in (("w", c["w"]), ("nx", g["nx"]), ("ny", g["ny"]), ("vol", g["vol"]),
                                       ("volf", g["volf"]), ("field", c["field"]), ("wbd", c["wbd"]), ("coef", coef))}
    cap = nrow * 245
    ip0 = torch.empty(nrow + 1, dtype=torch.int32, device="cuda")
    ix0 = torch.empty(cap, dtype=torch.int32, device="cuda")
    d0 = torch.empty(cap, dtype=torch.float64, device="cuda")
    nnz = run(plain, ip0, ix0, d0, cap)
    G = {k: Guarded(v) for k, v in (("w", c["w"]), ("nx", g["nx"]), ("ny", g["ny"]), ("vol", g["vol"]),
                                    ("volf", g["volf"]), ("field", c["field"]), ("wbd", c["wbd"]), ("coef", coef))}
    O = {"indptr": Guarded(shape=(nrow + 1,), dtype=np.int32), "indices": Guarded(shape=(nnz,), dtype=np.int32),
         "data": Guarded(shape=(nnz,))}
    assert run({k: v.flat for k, v in G.items()}, O["indptr"].flat, O["indices"].flat, O["data"].flat, nnz) == nnz
    _check(G)
    _check(O)
    assert np.array_equal(O["indptr"].flat.cpu().numpy(), ip0.cpu().numpy())
    assert np.array_equal(O["indices"].flat.cpu().numpy(), ix0[:nnz].cpu().numpy())
    assert np.array_equal(O["data"].flat.cpu().numpy(), d0[:nnz].cpu().numpy())
    # one entry short: the count is reported, nothing is written past the capacity
    S = {"indices": Guarded(shape=(nnz - 1,), dtype=np.int32), "data": Guarded(shape=(nnz - 1,))}
    with pytest.raises(_lib.BroadcastError):
        run({k: v.flat for k, v in G.items()}, O["indptr"].flat, S["indices"].flat, S["data"].flat, nnz - 1)
    _check(S)
    # spanwise operators
    wd = np.asfortranarray(np.random.default_rng(4).standard_normal(c["w"].shape))
    phs = [float(ph[k]) for k in KEYS[:9]]
    for name in ("bcg_coeffs_5p_dz", "bcg_coeffs_5p_dz2"):
        Z = {"out": Guarded(shape=c["w"].shape, fill=9.0), "wd": Guarded(wd)}
        _lib.call(name, Z["out"].flat, G["w"].flat, Z["wd"].flat, None, None, G["nx"].flat, G["ny"].flat, None, None,
                  G["vol"].flat, G["volf"].flat, gh, *phs, im, jm)
        _check(Z)
        _check(G)
        out = _plain(np.full(c["w"].shape, 9.0))
        _lib.call(name, out, plain["w"], _plain(wd), None, None, plain["nx"], plain["ny"], None, None, plain["vol"],
                  plain["volf"], gh, *phs, im, jm)
        z = Z["out"].host()
        assert np.isfinite(z).all()
        assert np.array_equal(z, np.reshape(out.cpu().numpy(), c["w"].shape, order="F"))


def test_krylov_solve():
    import torch
    from broadcast_gb300 import _lib
    from tests.test_gpu_linsolve import _banded
    A = _banded(700, 21, 14, seed=3, swapped=True)
    A.sort_indices()
    b = np.random.default_rng(2).standard_normal(700)
    G = {"indptr": Guarded(A.indptr.astype(np.int32)), "indices": Guarded(A.indices.astype(np.int32)),
         "data": Guarded(A.data), "b": Guarded(b), "x": Guarded(shape=(700,))}
    h, info = np.zeros(1, np.int64), np.zeros(1, np.int32)
    _lib.call("bcg_set_stream", torch.cuda.current_stream().cuda_stream)
    _lib.call("bcg_band32_factor", 700, G["indptr"].flat, G["indices"].flat, G["data"].flat, None, 32, h, info)
    try:
        it, rr = np.zeros(1, np.int32), np.zeros(1)
        _lib.call("bcg_gmres_solve", int(h[0]), 700, G["indptr"].flat, G["indices"].flat, G["data"].flat, G["b"].flat,
                  G["x"].flat, 30, 100, 1e-12, it, rr)
        _check(G)
        x = G["x"].host()
        assert np.isfinite(x).all() and np.linalg.norm(A @ x - b) <= 1e-11 * np.linalg.norm(b)
    finally:
        _lib.call("bcg_band32_destroy", int(h[0]))
