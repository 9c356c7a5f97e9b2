"""Spanwise operators Dz and Dzz (srcfv/dz/coeffs_5p_dz.F90, coeffs_5p_dz2.F90)
on the GPU against the oracle: several directions per call, both grid
families, device-resident arrays, and the batched Dz / Dzz CSR against the
reference's per-seed loop (BROADCAST_npz.py:1221-1249) run through the oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu
SPAN = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth")
TOL = 1e-12


def _dirs(c, nd, seed):
    rng = np.random.default_rng(seed)
    sc = np.abs(c["w"]).reshape(-1, 5).max(0)
    return np.stack([np.asfortranarray(rng.standard_normal(c["w"].shape) * sc) for _ in range(nd)])


def _span_args(c):
    g, ph = c["grid"], c["phys"]
    return (None, None, g["nx"], g["ny"], None, None, g["vol"], None, g["gh"]) + tuple(float(ph[k]) for k in SPAN) + (
        g["im"], g["jm"])


@pytest.mark.parametrize("kind,im,jm", [("bl", 40, 30), ("cyl", 64, 48)])
@pytest.mark.parametrize("op", ["dz", "dzz"])
@pytest.mark.parametrize("nd", [1, 3, 7])
def test_span_multi_direction_matches_oracle(kind, im, jm, op, nd):
    from broadcast_gb300 import _lib
    c = H.bl_case(im, jm) if kind == "bl" else H.cyl_case(im, jm)
    H.oracle_bcs(c, c["w"])
    wd = _dirs(c, nd, 11 + nd)
    ref = (O.dz if op == "dz" else O.dzz)(c["grid"], c["phys"], c["w"], wd)
    buf = np.asfortranarray(np.concatenate([np.ravel(x, order="F") for x in wd]))
    out = np.zeros_like(buf)
    _lib.call("bcg_coeffs_5p_dz_dn" if op == "dz" else "bcg_coeffs_5p_dz2_dn", out, c["w"], buf, nd, *_span_args(c))
    n = c["w"].size
    for k in range(nd):
        got = np.reshape(out[k * n:(k + 1) * n], c["w"].shape, order="F")
        sc = np.maximum(np.abs(H.interior(ref[k])).reshape(-1, 5).max(0), 1e-300)
        assert (np.abs(H.interior(got) - H.interior(ref[k])).reshape(-1, 5).max(0) / sc).max() < TOL


def test_span_on_device_tensors_is_linear():
    """Device arrays in place; Dz(a x + b y) = a Dz x + b Dz y to rounding."""
    import torch
    from broadcast_gb300 import _lib
    from broadcast_gb300.operator import to_device, to_host
    c = H.cyl_case(96, 64)
    H.oracle_bcs(c, c["w"])
    g = c["grid"]
    x, y = _dirs(c, 2, 5)
    dev = {k: to_device(g[k]) for k in ("nx", "ny", "vol")}
    w = to_device(c["w"])
    args = lambda: (None, None, dev["nx"], dev["ny"], None, None, dev["vol"], None, g["gh"]) + tuple(
        float(c["phys"][k]) for k in SPAN) + (g["im"], g["jm"])
    outs = []
    for v in (x, y, 2.0 * x - 3.0 * y):
        o = torch.zeros_like(w)
        _lib.call("bcg_coeffs_5p_dz", o, w, to_device(np.asfortranarray(v)), *args())
        outs.append(to_host(o))
    torch.cuda.synchronize()
    comb = 2.0 * outs[0] - 3.0 * outs[1]
    sc = np.abs(H.interior(comb)).reshape(-1, 5).max(0)
    assert (np.abs(H.interior(outs[2] - comb)).reshape(-1, 5).max(0) / sc).max() < 1e-12


def _reference_dz_csr(c, which, mini=2e-16):
    sp = pytest.importorskip("scipy.sparse")
    g = c["grid"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    nb = im * jm * 49 * 25
    jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
    fn = O.dz if which == 1 else O.dzz
    for m in range(5):
        for l in range(7):
            for k in range(7):
                wd = O.testvector(m, l, k, gh, im, jm)
                wtmp = c["w"].copy(order="F")
                H.oracle_bcs(c, wtmp, wd)
                out = fn(g, c["phys"], c["w"], wd)
                O.computejacobian(O.JAC_DZ, jac, ia, ja, out, m, l, k, gh, im, jm, None)
    keep = np.abs(jac) > mini
    a = sp.csr_matrix((jac[keep], (ia[keep], ja[keep])), shape=(5 * im * jm, 5 * im * jm))
    a.sum_duplicates()
    a.sort_indices()
    return a


@pytest.mark.parametrize("which", [1, 2])
def test_batched_dz_csr_matches_reference_loop(which):
    sp = pytest.importorskip("scipy.sparse")
    from broadcast_gb300 import _lib
    from broadcast_gb300._f2py import interf4
    c = H.bl_case(20, 14)
    H.oracle_bcs(c, c["w"])
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    nrow = 5 * im * jm
    cap = nrow * 245
    indptr, indices, data = np.zeros(nrow + 1, np.int32), np.zeros(cap, np.int32), np.zeros(cap)
    nnz = np.zeros(1, np.int64)
    _lib.call("bcg_jacobian_dz_bl_csr", c["w"], g["nx"], g["ny"], g["vol"], g["volf"], gh,
              *[float(ph[k]) for k in SPAN], im, jm, interf4(it["Ilo"]), interf4(it["Jhi"]), interf4(it["Ihi"]),
              interf4(it["Jlo"]), c["field"], c["field"].shape[0], c["wbd"], c["wbd"].shape[0], which, 2e-16,
              indptr, indices, data, cap, nnz)
    n = int(nnz[0])
    got = sp.csr_matrix((data[:n], indices[:n], indptr), shape=(nrow, nrow))
    ref = _reference_dz_csr(c, which)
    assert np.array_equal(got.indptr, ref.indptr)
    assert np.array_equal(got.indices, ref.indices)
    assert np.abs(got.data - ref.data).max() <= 1e-12 * np.abs(ref.data).max()


def _gpu_csr(c, fn, *extra):
    sp = pytest.importorskip("scipy.sparse")
    from broadcast_gb300 import _lib
    from broadcast_gb300._f2py import interf4
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    nrow = 5 * im * jm
    cap = nrow * 245
    indptr, indices, data = np.zeros(nrow + 1, np.int32), np.zeros(cap, np.int32), np.zeros(cap)
    nnz = np.zeros(1, np.int64)
    if fn == "jac":
        keys = SPAN + ("k2", "k4")
        _lib.call("bcg_jacobian_dnc5_bl_csr", c["w"], g["nx"], g["ny"], g["vol"], g["volf"], gh,
                  *[float(ph[k]) for k in keys], im, jm, interf4(it["Ilo"]), interf4(it["Jhi"]), interf4(it["Ihi"]),
                  interf4(it["Jlo"]), c["field"], c["field"].shape[0], c["wbd"], c["wbd"].shape[0], None, 2e-16, 1,
                  indptr, indices, data, cap, nnz)
    else:
        _lib.call("bcg_jacobian_dz_bl_csr", c["w"], g["nx"], g["ny"], g["vol"], g["volf"], gh,
                  *[float(ph[k]) for k in SPAN], im, jm, interf4(it["Ilo"]), interf4(it["Jhi"]), interf4(it["Ihi"]),
                  interf4(it["Jlo"]), c["field"], c["field"].shape[0], c["wbd"], c["wbd"].shape[0], extra[0], 2e-16,
                  indptr, indices, data, cap, nnz)
    n = int(nnz[0])
    return sp.csr_matrix((data[:n].copy(), indices[:n].copy(), indptr.copy()), shape=(nrow, nrow))


def test_spanwise_beta_operator():
    """J(beta) = Jacvol - beta^2 Dzz + i beta Dz (biglobal.py:82) on the union pattern."""
    from broadcast_gb300 import _lib
    c = H.bl_case(20, 14)
    H.oracle_bcs(c, c["w"])
    J, Dz, Dzz = _gpu_csr(c, "jac"), _gpu_csr(c, "dz", 1), _gpu_csr(c, "dz", 2)
    nrow = J.shape[0]
    betas = np.array([0.0, 0.4, 1.7])
    cap = J.nnz + Dz.nnz + Dzz.nnz
    indptr, indices = np.zeros(nrow + 1, np.int32), np.zeros(cap, np.int32)
    vals = np.zeros(2 * len(betas) * cap)
    nnz = np.zeros(1, np.int64)
    _lib.call("bcg_csr_spanwise_beta", nrow, J.indptr, J.indices, J.data, Dz.indptr, Dz.indices, Dz.data,
              Dzz.indptr, Dzz.indices, Dzz.data, len(betas), betas, indptr, indices, vals, cap, nnz)
    n = int(nnz[0])
    union = (abs(J) + abs(Dz) + abs(Dzz)).tocsr()
    union.sort_indices()
    assert n == union.nnz
    assert np.array_equal(indptr, union.indptr) and np.array_equal(indices[:n], union.indices)
    cv = vals[:2 * len(betas) * n].reshape(len(betas), n, 2)
    for k, b in enumerate(betas):
        got = (cv[k, :, 0] + 1j * cv[k, :, 1])
        ref = (J - b * b * Dzz + 1j * b * Dz).toarray()[np.repeat(np.arange(nrow), np.diff(indptr)), indices[:n]]
        assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()


@pytest.mark.parametrize("im,jm", [(20, 14), (64, 48)])
def test_one_pass_jacobian_dz_dzz_and_beta(im, jm):
    """bcg_jacobian_span_bl_csr (J/vol, Dz, Dzz from one seed loop, then J(beta))
    gives bit for bit what the three separate assemblies and
    bcg_csr_spanwise_beta give."""
    import torch
    sp = pytest.importorskip("scipy.sparse")
    from broadcast_gb300 import _lib
    from broadcast_gb300._f2py import interf4
    c = H.bl_case(im, jm)
    H.oracle_bcs(c, c["w"])
    g, ph, it = c["grid"], c["phys"], c["interf"]
    gh = g["gh"]
    J, Dz, Dzz = _gpu_csr(c, "jac"), _gpu_csr(c, "dz", 1), _gpu_csr(c, "dz", 2)
    nrow = 5 * im * jm
    cap = nrow * 245
    dev = torch.device("cuda", 0)
    outs = [(torch.zeros(nrow + 1, dtype=torch.int32, device=dev), torch.zeros(cap, dtype=torch.int32, device=dev),
             torch.zeros(cap, dtype=torch.float64, device=dev)) for _ in range(3)]
    tab = [np.array([o[k].data_ptr() for o in outs], np.uint64) for k in range(3)]
    caps, nnz3 = np.full(3, cap, np.int64), np.zeros(3, np.int64)
    betas = np.array([0.0, 0.4, 1.7])
    bcap = 3 * cap
    bp, bi = torch.zeros(nrow + 1, dtype=torch.int32, device=dev), torch.zeros(bcap, dtype=torch.int32, device=dev)
    bv, bn = torch.zeros(2 * len(betas) * bcap, dtype=torch.float64, device=dev), np.zeros(1, np.int64)
    keys = SPAN + ("k2", "k4")
    _lib.call("bcg_set_stream", torch.cuda.current_stream(dev).cuda_stream)
    _lib.call("bcg_jacobian_span_bl_csr", c["w"], g["nx"], g["ny"], g["vol"], g["volf"], gh,
              *[float(ph[k]) for k in keys], im, jm, interf4(it["Ilo"]), interf4(it["Jhi"]), interf4(it["Ihi"]),
              interf4(it["Jlo"]), c["field"], c["field"].shape[0], c["wbd"], c["wbd"].shape[0], 2e-16, 1,
              tab[0], tab[1], tab[2], caps, nnz3, len(betas), betas, bp, bi, bv, bcap, bn)
    torch.cuda.synchronize()
    for (p, i, v), ref, n in zip(outs, (J, Dz, Dzz), nnz3):
        assert n == ref.nnz
        assert np.array_equal(p.cpu().numpy(), ref.indptr)
        assert np.array_equal(i[:n].cpu().numpy(), ref.indices)
        assert np.array_equal(v[:n].cpu().numpy(), ref.data)
    # the epilogue against the separate call on the three host matrices
    rp, ri = np.zeros(nrow + 1, np.int32), np.zeros(bcap, np.int32)
    rv, rn = np.zeros(2 * len(betas) * bcap), np.zeros(1, np.int64)
    _lib.call("bcg_csr_spanwise_beta", nrow, J.indptr, J.indices, J.data, Dz.indptr, Dz.indices, Dz.data,
              Dzz.indptr, Dzz.indices, Dzz.data, len(betas), betas, rp, ri, rv, bcap, rn)
    n = int(rn[0])
    assert int(bn[0]) == n
    assert np.array_equal(bp.cpu().numpy(), rp) and np.array_equal(bi[:n].cpu().numpy(), ri[:n])
    assert np.array_equal(bv[:2 * len(betas) * n].cpu().numpy(), rv[:2 * len(betas) * n])
