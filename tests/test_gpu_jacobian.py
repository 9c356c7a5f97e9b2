"""Batched colored Jacobian assembly (all 245 seeds, CSR) against the
reference's per-seed loop (BROADCAST_npz.py:1068-1137) run through the
oracle: testvector, linearised boundary chain, tangent residual, COO fill,
remove_zero_jac, COO -> CSR.  The pattern must agree exactly and the values
within 1e-11 of the largest entry."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu
sp = pytest.importorskip("scipy.sparse")


def _reference_csr(c, coefdiag, mini=2e-16, divide_by_vol=False):
    g, ph = c["grid"], c["phys"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    nb = im * jm * 49 * 25
    jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
    for m in range(5):
        for l in range(7):
            for k in range(7):
                wd = O.testvector(m, l, k, gh, im, jm)
                wtmp = c["w"].copy(order="F")
                H.oracle_bcs(c, wtmp, wd)
                _, resd = O.jvp(g, ph, c["w"], wd)
                O.computejacobian(O.JAC_RELAXED if coefdiag is not None else O.JAC_PLAIN, jac, ia, ja, resd, m, l, k,
                                  gh, im, jm, coefdiag)
    keep = np.abs(jac) > mini
    jac, ia, ja = jac[keep], ia[keep], ja[keep]
    if divide_by_vol:
        vol = g["vol"]
        jac = jac / vol[(ia // (jm * 5)) + gh, ((ia % (jm * 5)) // 5) + gh]
    a = sp.csr_matrix((jac, (ia, ja)), shape=(5 * im * jm, 5 * im * jm))
    a.sum_duplicates()
    a.sort_indices()
    return a


def _gpu_csr(c, coefdiag, mini=2e-16, divide_by_vol=False):
    from broadcast_gb300 import _lib
    from broadcast_gb300._f2py import interf4
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    nrow = 5 * im * jm
    cap = nrow * 245
    indptr, indices, data = np.zeros(nrow + 1, np.int32), np.zeros(cap, np.int32), np.zeros(cap)
    nnz = np.zeros(1, np.int64)
    keys = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")
    _lib.call("bcg_jacobian_dnc5_bl_csr", c["w"], g["nx"], g["ny"], g["vol"], g["volf"], gh,
              *[float(ph[k]) for k in keys], im, jm, interf4(it["Ilo"]), interf4(it["Jhi"]), interf4(it["Ihi"]),
              interf4(it["Jlo"]), c["field"], c["field"].shape[0], c["wbd"], c["wbd"].shape[0],
              None if coefdiag is None else np.asfortranarray(coefdiag), mini, int(divide_by_vol), indptr, indices,
              data, cap, nnz)
    n = int(nnz[0])
    return sp.csr_matrix((data[:n], indices[:n], indptr), shape=(nrow, nrow))


@pytest.mark.parametrize("relaxed,divide", [(True, False), (False, True)])
def test_batched_jacobian_matches_reference_loop(relaxed, divide):
    c = H.bl_case(20, 14)
    H.oracle_bcs(c, c["w"])
    coef = np.asfortranarray(np.random.default_rng(9).uniform(0.5, 2.0, (20, 14))) if relaxed else None
    ref = _reference_csr(c, coef, divide_by_vol=divide)
    got = _gpu_csr(c, coef, divide_by_vol=divide)
    assert np.array_equal(got.indptr, ref.indptr)
    assert np.array_equal(got.indices, ref.indices)
    scale = np.abs(ref.data).max()
    assert np.abs(got.data - ref.data).max() <= 1e-11 * scale


def test_batched_jacobian_columns_against_dense_jvp():
    """Every column of the assembled Jacobian equals a single-cell JVP."""
    c = H.bl_case(14, 10)
    H.oracle_bcs(c, c["w"])
    got = _gpu_csr(c, None, mini=-1.0).toarray()   # keep every candidate entry
    g, ph = c["grid"], c["phys"]
    rng = np.random.default_rng(3)
    for col in rng.choice(5 * 14 * 10, size=12, replace=False):
        m, jj, ii = col % 5, (col // 5) % 10, col // 50
        wd = np.zeros_like(c["w"])
        wd[ii + 3, jj + 3, m] = 1.0
        wtmp = c["w"].copy(order="F")
        H.oracle_bcs(c, wtmp, wd)
        _, resd = O.jvp(g, ph, c["w"], wd)
        dense = -np.transpose(H.interior(resd), (0, 1, 2)).reshape(-1)  # (i, j, e) C order = row numbering
        assert np.abs(got[:, col] - dense).max() <= 1e-11 * max(1.0, np.abs(dense).max())


def _reference_cyl_csr(c, coefdiag, mini=2e-16):
    """The cylinder driver's loop (cylinder.py:899-980): for im a multiple of
    7, testvector and computejacobianfromjv[_relaxed]_withjn; otherwise two
    azimuthal zones (Nzones: columns below and from im/2/7*7), testvector_partial
    and computejacobianfromjv_relaxed_withjnandcheck per zone (its plain form
    with a zero coefdiag)."""
    g = c["grid"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    zoned = im % 7 != 0
    nb = im * jm * 49 * 25 * (2 if zoned else 1)
    jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
    mode = O.JAC_RELAXED_WITHJN if coefdiag is not None else O.JAC_WITHJN
    imid = im // 2 // 7 * 7
    zones = [(0, imid - 1), (imid, im - 1)] if zoned else [None]
    cd = coefdiag if coefdiag is not None else np.zeros((im, jm), order="F")
    for n, zone in enumerate(zones):
        for m in range(5):
            for l in range(7):
                for k in range(7):
                    if zone is None:
                        wd = O.testvector(m, l, k, gh, im, jm)
                    else:
                        wd = O.testvector_partial(m, l, k, gh, im, jm, zone[0], zone[1], 0, jm - 1)
                    H.oracle_bcs(c, c["w"].copy(order="F"), wd)
                    _, resd = O.jvp(g, c["phys"], c["w"], wd)
                    if zone is None:
                        O.computejacobian(mode, jac, ia, ja, resd, m, l, k, gh, im, jm, coefdiag)
                    else:
                        O.computejacobian_withjnandcheck(jac, ia, ja, resd, m, l, k, gh, im, jm, cd, mini, n)
    keep = np.abs(jac) > mini
    a = sp.csr_matrix((jac[keep], (ia[keep], ja[keep])), shape=(5 * im * jm, 5 * im * jm))
    a.sum_duplicates()
    a.sort_indices()
    return a


@pytest.mark.parametrize("im,relaxed", [(21, True), (20, False), (22, True)])
def test_batched_cylinder_jacobian_matches_reference_loop(im, relaxed):
    """Periodic O-mesh: joins in the tangent chain, columns wrapped in i
    (computejacobianfromjv[_relaxed]_withjn); when im is not a multiple of 7
    the driver's two azimuthal zones of seeds."""
    from broadcast_gb300 import _lib
    from broadcast_gb300._f2py import interf4
    c = H.cyl_case(im, 10)
    H.oracle_bcs(c, c["w"])
    g, ph, it = c["grid"], c["phys"], c["interf"]
    jm, gh = g["jm"], g["gh"]
    coef = np.asfortranarray(np.random.default_rng(2).uniform(0.5, 2.0, (im, jm))) if relaxed else None
    ref = _reference_cyl_csr(c, coef)
    nrow = 5 * im * jm
    cap = nrow * 245
    indptr, indices, data = np.zeros(nrow + 1, np.int32), np.zeros(cap, np.int32), np.zeros(cap)
    nnz = np.zeros(1, np.int64)
    keys = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")
    pr = lambda a: interf4(a)
    _lib.call("bcg_jacobian_dnc5_cyl_csr", c["w"], g["nx"], g["ny"], g["vol"], g["volf"], gh,
              *[float(ph[k]) for k in keys], im, jm, pr(it["Jhi"]), pr(it["Jlo"]), c["wbd"], c["wbd"].shape[0],
              pr(it["prr1"]), pr(it["prd1"]), pr(it["prr2"]), pr(it["prd2"]),
              np.ascontiguousarray(np.asarray(it["tr"], dtype=np.int32).ravel()), coef, 2e-16, 0, indptr, indices,
              data, cap, nnz)
    n = int(nnz[0])
    got = sp.csr_matrix((data[:n], indices[:n], indptr), shape=(nrow, nrow))
    assert np.array_equal(got.indptr, ref.indptr)
    assert np.array_equal(got.indices, ref.indices)
    assert np.abs(got.data - ref.data).max() <= 1e-11 * np.abs(ref.data).max()


def test_cylinder_jacobian_columns_at_the_periodic_join():
    """im = 22 (not a multiple of 7): the columns of the assembled periodic
    Jacobian next to the join, where one colour's seeds of a single zone would
    meet across it, equal single-cell tangents (seed, tangent fills with the
    joins, flux_num_dnc5_2d_d)."""
    from broadcast_gb300 import _lib
    from broadcast_gb300._f2py import interf4
    im, jm = 22, 10
    c = H.cyl_case(im, jm)
    H.oracle_bcs(c, c["w"])
    g, ph, it = c["grid"], c["phys"], c["interf"]
    gh = g["gh"]
    nrow = 5 * im * jm
    cap = nrow * 245
    indptr, indices, data = np.zeros(nrow + 1, np.int32), np.zeros(cap, np.int32), np.zeros(cap)
    nnz = np.zeros(1, np.int64)
    keys = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")
    pr = interf4
    _lib.call("bcg_jacobian_dnc5_cyl_csr", c["w"], g["nx"], g["ny"], g["vol"], g["volf"], gh,
              *[float(ph[k]) for k in keys], im, jm, pr(it["Jhi"]), pr(it["Jlo"]), c["wbd"], c["wbd"].shape[0],
              pr(it["prr1"]), pr(it["prd1"]), pr(it["prr2"]), pr(it["prd2"]),
              np.ascontiguousarray(np.asarray(it["tr"], dtype=np.int32).ravel()), None, 2e-16, 0, indptr, indices,
              data, cap, nnz)
    n = int(nnz[0])
    got = sp.csr_matrix((data[:n], indices[:n], indptr), shape=(nrow, nrow)).toarray()
    for ii in (0, 1, 2, im - 3, im - 2, im - 1):
        for jj in (0, 4):
            for mm in (0, 3):
                col = mm + 5 * jj + 5 * jm * ii
                wd = np.zeros_like(c["w"])
                wd[ii + gh, jj + gh, mm] = 1.0
                H.oracle_bcs(c, c["w"].copy(order="F"), wd)
                _, resd = O.jvp(g, ph, c["w"], wd)
                dense = -H.interior(resd).reshape(-1)  # (i, j, e) C order = row numbering
                assert np.abs(got[:, col] - dense).max() <= 1e-11 * max(1.0, np.abs(dense).max()), (ii, jj, mm)
