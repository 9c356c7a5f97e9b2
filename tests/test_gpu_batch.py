"""Uneven batch of boundary-layer grids (broadcast_gb300.batch, bcg_batch_*):
per-instance residual and tangent against the single-grid kernels and the
oracle, graph replay with new array addresses, every tile configuration, and
the autotuner's cache."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import helpers as H

pytestmark = pytest.mark.gpu


def _cases(n=5, seed=4):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        im, jm = int(rng.integers(20, 90)), int(rng.integers(10, 40))
        c = H.bl_case(im, jm, mach=float(rng.uniform(0.3, 0.8)), seed=k)
        H.oracle_bcs(c, c["w"])
        wd = np.zeros_like(c["w"])
        wd[3:-3, 3:-3] = rng.standard_normal((im, jm, 5))
        H.oracle_bcs(c, c["w"].copy(order="F"), wd)
        out.append((c, wd))
    return out


def _batch(cases, ndir=1):
    from broadcast_gb300.batch import GridBatch
    from broadcast_gb300.operator import to_device
    gb = GridBatch([c["grid"] for c, _ in cases], [c["phys"] for c, _ in cases], ndir=ndir)
    gb.set_states([to_device(c["w"]) for c, _ in cases], [to_device(wd) for _, wd in cases] if ndir else None)
    return gb


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_matches_single_grid_and_oracle(use_graph):
    import torch
    from broadcast_gb300.operator import Dnc5Operator, to_device, to_host
    cases = _cases()
    gb = _batch(cases)
    gb.run(use_graph=use_graph)
    torch.cuda.synchronize()
    for g, (c, wd) in enumerate(cases):
        op = Dnc5Operator(c["grid"], c["phys"])
        r1, rd1 = op.jvp(to_device(c["w"]), to_device(wd))
        r, rd = to_host(gb.res[g]), to_host(gb.resd[g])
        sc = H.flux_scale(c, c["w"])
        assert H.rel_err(r, to_host(r1), sc) < 1e-13
        ref, refd = O.jvp(c["grid"], c["phys"], c["w"], wd)
        assert H.rel_err(r, ref, sc) < 1e-12
        scd = np.abs(H.interior(refd)).reshape(-1, 5).max(0)
        assert H.rel_err(rd, refd, scd) < 1e-11
        assert H.rel_err(rd, to_host(rd1), scd) < 1e-13


def test_graph_replay_follows_new_arrays_and_every_tile_shape():
    import torch
    from broadcast_gb300.batch import CANDIDATES
    from broadcast_gb300.operator import to_device, to_host
    cases = _cases(4, seed=9)
    gb = _batch(cases)
    gb.run(use_graph=True)
    torch.cuda.synchronize()
    first = [to_host(r).copy() for r in gb.res]
    # new states (different noise) through the same captured graph
    cases2 = [(dict(c, w=c["w"] * 1.0001), wd) for c, wd in cases]
    gb.set_states([to_device(c["w"]) for c, _ in cases2], [to_device(wd) for _, wd in cases2])
    gb.run(use_graph=True)
    torch.cuda.synchronize()
    for g, (c, _) in enumerate(cases2):
        ref = O.residual(c["grid"], c["phys"], c["w"])
        assert H.rel_err(to_host(gb.res[g]), ref, H.flux_scale(c, c["w"])) < 1e-12
        assert not np.array_equal(to_host(gb.res[g]), first[g])
    for cand in CANDIDATES:
        gb.configure(*cand)
        gb.run(use_graph=False)
        torch.cuda.synchronize()
        for g, (c, _) in enumerate(cases2):
            ref = O.residual(c["grid"], c["phys"], c["w"])
            assert H.rel_err(to_host(gb.res[g]), ref, H.flux_scale(c, c["w"])) < 1e-12, cand


def test_residual_only_batch_and_autotune_cache(tmp_path):
    import torch
    from broadcast_gb300.operator import to_host
    cases = _cases(3, seed=2)
    gb = _batch(cases, ndir=0)
    cache = str(tmp_path / "tune.json")
    entry = gb.autotune(repeats=2, cache=cache)
    assert tuple(entry["config"]) == gb.config and len(entry["timings"]) > 4
    again = gb.autotune(cache=cache)  # served from the cache
    assert again["config"] == entry["config"]
    gb.run(use_graph=True)
    torch.cuda.synchronize()
    for g, (c, _) in enumerate(cases):
        ref = O.residual(c["grid"], c["phys"], c["w"])
        assert H.rel_err(to_host(gb.res[g]), ref, H.flux_scale(c, c["w"])) < 1e-12


def test_full_size_uneven_grids_at_the_sensor_tie():
    """Two full-size grids of the 64-grid uneven batch (933x294 and 353x294)
    whose outflow column i = im holds a face where the pressure sensor's two
    ratios agree to ~1e-7 (second differences ~8e-10 of p ~ 1.2 next to the
    linearly extrapolated ghosts): MAX(ks1, ks2) there follows the pressure's
    last bits.  Every interior cell of the tangent, i = im included, within
    1e-11 of max|R'v| of the oracle, through the single-grid operator and the
    batch."""
    import torch
    from broadcast_gb300 import cases
    from broadcast_gb300.batch import GridBatch
    from broadcast_gb300.operator import Dnc5Operator, to_device, to_host
    sel = []
    for k, c, wd in cases.uneven_bl_batch(only=(8, 29), ops=H.OracleOps):
        H.oracle_bcs(c, c["w"])
        sel.append((c, wd))
    assert [c["grid"]["im"] for c, _ in sel] == [933, 353]
    gb = GridBatch([c["grid"] for c, _ in sel], [c["phys"] for c, _ in sel], ndir=1)
    gb.set_states([to_device(c["w"]) for c, _ in sel], [to_device(wd) for _, wd in sel])
    gb.run(use_graph=True)
    torch.cuda.synchronize()
    for g, (c, wd) in enumerate(sel):
        ref, refd = O.jvp(c["grid"], c["phys"], c["w"], wd)
        scd = np.abs(H.interior(refd)).reshape(-1, 5).max(0)
        op = Dnc5Operator(c["grid"], c["phys"])
        r1, rd1 = op.jvp(to_device(c["w"]), to_device(wd))
        for rd in (to_host(rd1), to_host(gb.resd[g])):
            cell = (np.abs(H.interior(rd) - H.interior(refd)) / scd).max(axis=2)
            assert cell.max() < 1e-11, (g, cell.max(), np.unravel_index(cell.argmax(), cell.shape))
        assert H.rel_err(to_host(r1), ref, H.flux_scale(c, c["w"])) < 1e-12


@pytest.mark.parametrize("nchunk", [1, 3, 16])
def test_host_array_run_matches_device_run(nchunk):
    """bcg_batch_run_host: host arrays in, overlapped chunk uploads / graph
    replays / interior downloads, the same results as the device-array run
    bit for bit, and the caller's ghost values of residu and residud kept."""
    import torch
    from broadcast_gb300.operator import to_host
    cases = _cases(6, seed=11)
    gb = _batch(cases)
    gb.run(use_graph=True)
    torch.cuda.synchronize()
    ref = [(to_host(r).copy(), to_host(rd).copy()) for r, rd in zip(gb.res, gb.resd)]
    res = [np.full_like(c["w"], 7.0) for c, _ in cases]
    resd = [np.full_like(c["w"], -3.0) for c, _ in cases]
    for _ in range(2):  # the second call reuses the plan's mirrors and chunk graphs
        gb.run_host([c["w"] for c, _ in cases], [wd for _, wd in cases], res, resd, [c["grid"] for c, _ in cases],
                    nchunk=nchunk)
        for g in range(len(cases)):
            assert np.array_equal(H.interior(res[g]), H.interior(ref[g][0]))
            assert np.array_equal(H.interior(resd[g]), H.interior(ref[g][1]))
            ghost = np.ones(res[g].shape, bool)
            ghost[3:-3, 3:-3] = False
            assert (res[g][ghost] == 7.0).all() and (resd[g][ghost] == -3.0).all()


def test_host_run_tile_shapes_of_their_own():
    """The chunks of host-array runs take tile shapes of their own
    (bcg_batch_configure_host, and the autotuner over them), which a later
    configure of the whole batch leaves alone; results bit for bit those of the
    device-array run under every shape."""
    import torch
    from broadcast_gb300.batch import CANDIDATES
    from broadcast_gb300.operator import to_host
    cases = _cases(5, seed=12)
    gb = _batch(cases)
    gb.configure(128, 256, 2)
    gb.run(use_graph=True)
    torch.cuda.synchronize()
    ref = [(to_host(r).copy(), to_host(rd).copy()) for r, rd in zip(gb.res, gb.resd)]
    ws, wds, geo = [c["w"] for c, _ in cases], [wd for _, wd in cases], [c["grid"] for c, _ in cases]
    res = [np.zeros_like(c["w"]) for c, _ in cases]
    resd = [np.zeros_like(c["w"]) for c, _ in cases]

    def same():
        for g in range(len(cases)):
            assert np.array_equal(H.interior(res[g]), H.interior(ref[g][0]))
            assert np.array_equal(H.interior(resd[g]), H.interior(ref[g][1]))

    gb.run_host(ws, wds, res, resd, geo, nchunk=3)
    same()
    for cand in CANDIDATES[::5]:
        gb.configure_host(*cand)
        gb.run_host(ws, wds, res, resd, geo, nchunk=3)
        same()
    gb.configure_host(64, 128, 4)
    gb.configure(256, 128, 1)  # the whole batch's shapes change, the chunks' stay
    gb.run_host(ws, wds, res, resd, geo, nchunk=3)
    same()
    tune = gb.autotune_host(ws, wds, res, resd, geo, nchunk=3, candidates=CANDIDATES[:4], repeats=1)
    assert tuple(tune["config"]) in CANDIDATES[:4] and gb.host_config == tuple(tune["config"])
    gb.run_host(ws, wds, res, resd, geo, nchunk=3)
    same()


def test_rectilinear_and_curvilinear_grids_in_one_graph():
    """Rectilinear boundary layers take the face kernel without the zero metric
    products, a curvilinear O-mesh the general one, in the same launch; the
    choice follows the metrics at every replay: a boundary layer whose one
    i-face normal gets a nonzero ny on the device is curvilinear at the next
    replay, and both grids still equal the oracle."""
    import torch
    from broadcast_gb300.operator import to_host
    rng = np.random.default_rng(7)
    cases = _cases(3, seed=9)
    c = H.cyl_case(40, 24)
    H.oracle_bcs(c, c["w"])
    wd = np.zeros_like(c["w"])
    wd[3:-3, 3:-3] = rng.standard_normal((40, 24, 5))
    H.oracle_bcs(c, c["w"].copy(order="F"), wd)
    cases.insert(1, (c, wd))
    gb = _batch(cases)

    def check():
        gb.run(use_graph=True)
        torch.cuda.synchronize()
        for g, (cc, wdd) in enumerate(cases):
            ref, refd = O.jvp(cc["grid"], cc["phys"], cc["w"], wdd)
            assert H.rel_err(to_host(gb.res[g]), ref, H.flux_scale(cc, cc["w"])) < 1e-12
            scd = np.abs(H.interior(refd)).reshape(-1, 5).max(0)
            assert H.rel_err(to_host(gb.resd[g]), refd, scd) < 1e-11

    check()
    g = 2
    cc = cases[g][0]
    bump = 1e-3 * np.abs(cc["grid"]["nx"][..., 0]).max()
    cc["grid"]["ny"][7, 6, 0] += bump      # Fortran (i, j, plane) on the host
    gb.geo[g]["ny"][0, 6, 7] += bump        # the same entry of the device tensor (plane, j, i)
    check()
