"""The batched colored Jacobian (bcg_jacobian_dnc5_bl_csr: all 245 seeds in
one call, CSR) at the sizes of the reference's configurations, against the
reference's per-seed loop run through the oracle (BROADCAST_npz.py:1068-1137:
testvector, the linearised boundary chain, flux_num_dnc5_2d_d,
computejacobianfromjv[_relaxed] (misc/ComputeJacobian.f90:292-355, 503-570),
remove_zero_jac with |a| > 2e-16 (BROADCAST_npz.py:129-135), Jac/vol
(:1206-1210)).

- 400x150 boundary layer (Newton's relaxed Jacobian): the whole CSR, pattern
  (indptr, indices) bit-exact and values within 1e-11 of the largest entry;
  the structural (pre-filter) pattern as well.
- 1024x512 boundary layer (the stability Jacobian J/vol): the full COO of
  the reference loop (642M slots) does not fit a test, so the loop runs seed
  by seed and keeps, per row, the counts of the structural and of the filtered
  pattern (= the whole indptr of both), and every entry of three bands of rows
  (inlet, middle, outflow); and J v against the oracle's JVP for random v.
  Filter decisions on cancellation residues near 2e-16 may differ between the
  two computations; they are bounded and counted.
Entries near the filter threshold (where a rounding difference could flip the
pattern) are counted and reported."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu
sp = pytest.importorskip("scipy.sparse")

KEYS = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")
MINI = 2e-16


def _gpu_csr(c, coefdiag, mini, divide_by_vol, cap):
    """The library's batched assembly into device arrays; returns (indptr,
    indices, data) as torch tensors on the device and nnz."""
    import torch
    from broadcast_gb300 import _lib
    from broadcast_gb300._f2py import interf4
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    nrow = 5 * im * jm
    dev = torch.device("cuda")
    indptr = torch.empty(nrow + 1, dtype=torch.int32, device=dev)
    indices = torch.empty(cap, dtype=torch.int32, device=dev)
    data = torch.empty(cap, dtype=torch.float64, device=dev)
    nnz = np.zeros(1, np.int64)
    _lib.call("bcg_set_stream", torch.cuda.current_stream().cuda_stream)
    _lib.call("bcg_jacobian_dnc5_bl_csr", c["w"], g["nx"], g["ny"], g["vol"], g["volf"], gh,
              *[float(ph[k]) for k in KEYS], im, jm, interf4(it["Ilo"]), interf4(it["Jhi"]), interf4(it["Ihi"]),
              interf4(it["Jlo"]), c["field"], c["field"].shape[0], c["wbd"], c["wbd"].shape[0],
              None if coefdiag is None else np.asfortranarray(coefdiag), mini, int(divide_by_vol), indptr, indices,
              data, cap, nnz)
    torch.cuda.synchronize()
    return indptr, indices, data, int(nnz[0])


def _seed_sweep(c, mode, coefdiag, visit, stack=8):
    """The reference loop seed by seed: testvector, the tangent boundary chain,
    the oracle's tangent (stacks of seeds, all host cores), and the COO slots
    of every output; visit(ia, ja, jac) per seed."""
    g, ph = c["grid"], c["phys"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    seeds = [(m, l, k) for m in range(5) for l in range(7) for k in range(7)]
    for s0 in range(0, len(seeds), stack):
        grp = seeds[s0:s0 + stack]
        wds = []
        for (m, l, k) in grp:
            wd = O.testvector(m, l, k, gh, im, jm)
            H.oracle_bcs(c, c["w"].copy(order="F"), wd)
            wds.append(wd)
        _, resd = O.jvp(g, ph, c["w"], np.stack(wds), openmp=True)
        for (m, l, k), rd in zip(grp, resd):
            visit(*O.computejacobian_band(mode, np.asfortranarray(rd), m, l, k, gh, im, jm, coefdiag))


def _valid(ia, ja, jac, bad):
    """Slots that hold an entry: the reference marks the others with row
    5 im jm - 1, column 0 and value 0 (that row is also the last cell's
    genuine row, whose entries never sit in column 0)."""
    return ~((ia == bad) & (ja == 0) & (jac == 0.0))


def _row_volume(c, ia):
    g = c["grid"]
    jm, gh = g["jm"], g["gh"]
    return g["vol"][(ia // (jm * 5)) + gh, ((ia % (jm * 5)) // 5) + gh]


def test_relaxed_jacobian_400x150_whole_csr():
    im, jm = 400, 150
    c = H.bl_case(im, jm, seed=0)
    H.oracle_bcs(c, c["w"])
    nrow = 5 * im * jm
    coef = np.asfortranarray(np.random.default_rng(9).uniform(0.5, 2.0, (im, jm)))
    bad = nrow - 1
    rows, cols, vals = [], [], []
    struct = np.zeros(nrow, np.int64)
    near = []

    def visit(ia, ja, jac):
        valid = _valid(ia, ja, jac, bad)
        struct[:] += np.bincount(ia[valid], minlength=nrow)
        keep = valid & (np.abs(jac) > MINI)
        rows.append(ia[keep]); cols.append(ja[keep]); vals.append(jac[keep])
        nb = valid & (np.abs(jac) > MINI / 4) & (np.abs(jac) < MINI * 4)
        near.extend(zip(ia[nb].tolist(), ja[nb].tolist(), jac[nb].tolist()))

    _seed_sweep(c, O.JAC_RELAXED, coef, visit)
    ref = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nrow, nrow))
    ref.sum_duplicates()
    ref.sort_indices()
    indptr, indices, data, nnz = _gpu_csr(c, coef, MINI, False, nrow * 245)
    got_ptr = indptr.cpu().numpy()
    assert np.array_equal(got_ptr, ref.indptr), "filtered pattern: row counts differ"
    assert np.array_equal(indices[:nnz].cpu().numpy(), ref.indices), "filtered pattern: columns differ"
    scale = np.abs(ref.data).max()
    err = np.abs(data[:nnz].cpu().numpy() - ref.data).max() / scale
    assert err <= 1e-11, err
    # structural pattern: every valid slot kept (mini < 0)
    sptr, _, _, snnz = _gpu_csr(c, coef, -1.0, False, nrow * 245)
    assert snnz == int(struct.sum())
    assert np.array_equal(np.diff(sptr.cpu().numpy()), struct)
    print("400x150 relaxed J: nnz %d (structural %d), max rel err %.2e, entries within 4x of 2e-16: %d %s"
          % (nnz, snnz, err, len(near), near[:10]))


def test_stability_jacobian_1024x512_indptr_bands_and_products():
    """J/vol of the 1024x512 boundary layer.  The structural pattern (every
    valid slot, before the |a| > 2e-16 filter) must be exact in every row, and
    on three bands of rows (inlet, middle, outflow) every entry's value within
    1e-11 of the largest.  After the filter, the row counts may differ only
    through entries that are cancellation residues -- exact zeros of the
    derivative rounded to ~1e-16 by each computation's own operation order,
    which the threshold 2e-16 (BROADCAST_npz.py:129-135) cuts through: each
    such flip is checked to be below 1e-13 of its row's largest entry in both
    computations, and the flips are counted."""
    import torch
    im, jm = 1024, 512
    c = H.bl_case(im, jm, seed=3)
    H.oracle_bcs(c, c["w"])
    g, ph = c["grid"], c["phys"]
    nrow = 5 * im * jm
    bad = nrow - 1
    bands = [(1, 8), (509, 516), (1017, 1024)]
    band_rows = [(5 * jm * (i0 - 1), 5 * jm * i1) for i0, i1 in bands]
    # the library: J/vol after the filter, and every valid slot (raw J) before it
    indptr, indices, data, nnz = _gpu_csr(c, None, MINI, True, nrow * 245)
    got_ptr = indptr.cpu().numpy().astype(np.int64)
    sptr_d, sidx_d, sdat_d, snnz = _gpu_csr(c, None, -1.0, False, nrow * 245)
    sptr = sptr_d.cpu().numpy().astype(np.int64)
    struct = np.zeros(nrow, np.int64)
    post = np.zeros(nrow, np.int64)
    csum = np.zeros(nrow)   # per row: sum of the kept columns and of their squares
    csq = np.zeros(nrow)
    picks = [([], [], []) for _ in bands]
    near = [0]

    def visit(ia, ja, jac):
        valid = _valid(ia, ja, jac, bad)
        struct[:] += np.bincount(ia[valid], minlength=nrow)
        keep = valid & (np.abs(jac) > MINI)
        post[:] += np.bincount(ia[keep], minlength=nrow)
        colk = ja[keep].astype(np.float64)
        csum[:] += np.bincount(ia[keep], weights=colk, minlength=nrow)
        csq[:] += np.bincount(ia[keep], weights=colk * colk, minlength=nrow)
        near[0] += int((valid & (np.abs(jac) > MINI / 4) & (np.abs(jac) < MINI * 4)).sum())
        for (r0, r1), (pr, pc, pv) in zip(band_rows, picks):
            sel = valid & (ia >= r0) & (ia < r1)
            pr.append(ia[sel]); pc.append(ja[sel]); pv.append(jac[sel])

    _seed_sweep(c, O.JAC_PLAIN, None, visit, stack=4)
    # structural pattern: exact in every row
    assert snnz == int(struct.sum())
    assert np.array_equal(np.diff(sptr), struct)
    # every entry of the three bands, before the filter
    scale, errs = 0.0, []
    for (r0, r1), (pr, pc, pv) in zip(band_rows, picks):
        ref = sp.csr_matrix((np.concatenate(pv), (np.concatenate(pr) - r0, np.concatenate(pc))), shape=(r1 - r0, nrow))
        ref.sum_duplicates()
        ref.sort_indices()
        a, b = int(sptr[r0]), int(sptr[r1])
        assert np.array_equal(sptr[r0:r1 + 1] - a, ref.indptr)
        assert np.array_equal(sidx_d[a:b].cpu().numpy(), ref.indices)
        scale = max(scale, np.abs(ref.data).max())
        errs.append(np.abs(sdat_d[a:b].cpu().numpy() - ref.data).max())
    band_err = max(errs) / scale
    assert band_err <= 1e-11, band_err
    # the filtered pattern: rows whose kept columns differ (count, sum, sum of
    # squares) hold only residue flips
    rid = torch.repeat_interleave(torch.arange(nrow, device=indptr.device), torch.diff(indptr.long()))
    colf = indices[:nnz].double()
    gsum = torch.zeros(nrow, dtype=torch.float64, device=indptr.device).index_add_(0, rid, colf).cpu().numpy()
    gsq = torch.zeros(nrow, dtype=torch.float64, device=indptr.device).index_add_(0, rid, colf * colf).cpu().numpy()
    del rid, colf
    rows = np.nonzero((np.diff(got_ptr) != post) | (gsum != csum) | (gsq != csq))[0]
    flips = []
    if rows.size:
        assert rows.size < 1e-4 * nrow, rows.size
        want = {int(r): {} for r in rows}
        rset = np.asarray(sorted(want))

        def collect(ia, ja, jac):
            sel = np.isin(ia, rset) & _valid(ia, ja, jac, bad)
            for r, col, v in zip(ia[sel].tolist(), ja[sel].tolist(), jac[sel].tolist()):
                want[r][col] = v

        _seed_sweep(c, O.JAC_PLAIN, None, collect, stack=4)
        for r, ora in want.items():
            a, b = int(sptr[r]), int(sptr[r + 1])
            mine = dict(zip(sidx_d[a:b].cpu().numpy().tolist(), sdat_d[a:b].cpu().numpy().tolist()))
            assert set(mine) == set(ora)
            rowmax = max(abs(v) for v in ora.values())
            kept_lib = set(indices[int(got_ptr[r]):int(got_ptr[r + 1])].cpu().numpy().tolist())
            assert kept_lib == {col for col, v in mine.items() if abs(v) > MINI}
            for col, v in ora.items():
                if (abs(v) > MINI) != (abs(mine[col]) > MINI):
                    assert max(abs(v), abs(mine[col])) <= 1e-13 * rowmax, (r, col, v, mine[col], rowmax)
                    flips.append((r, col, v, mine[col]))
        assert len(flips) >= 1
    del sidx_d, sdat_d
    torch.cuda.empty_cache()
    # J v against the oracle's tangent (the same linearised boundary chain)
    J = sp.csr_matrix((data[:nnz].cpu().numpy(), indices[:nnz].cpu().numpy(), got_ptr), shape=(nrow, nrow))
    rng = np.random.default_rng(12)
    for _ in range(2):
        v = rng.standard_normal((im, jm, 5))
        wd = np.zeros_like(c["w"])
        wd[3:-3, 3:-3] = v
        H.oracle_bcs(c, c["w"].copy(order="F"), wd)
        _, rd = O.jvp(g, ph, c["w"], wd, openmp=True)
        want_v = (-H.interior(rd) / H.interior(g["vol"])[:, :, None]).reshape(-1)  # (i, j, e) C order = row order
        err = np.abs(J @ v.reshape(-1) - want_v).max() / np.abs(want_v).max()
        assert err <= 1e-11, err
    print("1024x512 J/vol: nnz %d (structural %d), band max rel err %.2e, J v max rel err %.2e, entries within 4x of "
          "2e-16: %d, filter flips (residues < 1e-13 of the row): %d %s"
          % (nnz, snnz, band_err, err, near[0], len(flips), flips[:6]))
