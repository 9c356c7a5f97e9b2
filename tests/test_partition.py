"""Domain decomposition in i (broadcast_gb300.partition) on CPU ranks.

Ranks are gloo processes on 127.0.0.1.  Each rank takes its slab of a grid
whose ghost cells were filled by the drivers' boundary sequence, overwrites
its halo columns with NaN, exchanges halos, and evaluates the residual of its
slab (the oracle stands in for the GPU kernels here: the decomposition logic
is what is under test).  The owned columns must equal the single-grid
residual exactly, for the boundary-layer grid (open in i) and the periodic
O-mesh (first and last slab joined).  Failure cases: a rank that exits before
the exchange and a rank that stays alive but never sends both end in
HaloTimeout on its neighbour within the time limit.
"""
import datetime
import os
import socket
import tempfile
import time

import numpy as np
import pytest

from tests import helpers as H


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _init(rank, ws, port, timeout=20):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws, timeout=datetime.timedelta(seconds=timeout))
    return dist


def _case(kind):
    c = H.bl_case(40, 16) if kind == "bl" else H.cyl_case(36, 14)
    H.oracle_bcs(c, c["w"])
    return c


def _worker_residual(rank, ws, port, kind, outdir):
    from broadcast_gb300.partition import ColumnSlabs, HaloExchange, global_norml2
    from oracle import oracle as O
    dist = _init(rank, ws, port)
    c = _case(kind)
    g = c["grid"]
    slabs = ColumnSlabs(g["im"], g["jm"], ws, periodic=(kind == "cyl"))
    loc = slabs.extract_grid(g, rank)
    w = slabs.extract_cells(c["w"], rank).copy(order="F")
    halo = HaloExchange(slabs, rank, timeout=10.0)
    if halo.left is not None:
        w[:halo.width] = np.nan
    if halo.right is not None:
        w[-halo.width:] = np.nan
    halo.exchange(w)
    r = O.residual(loc, c["phys"], w)
    sumsq = (r[slabs.owned_slice(rank), 3:-3] ** 2).sum(axis=(0, 1))
    norm = global_norml2(sumsq)
    np.savez(os.path.join(outdir, "r%d.npz" % rank), r=r, norm=norm)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("kind,ws", [("bl", 2), ("cyl", 2), ("bl", 3), ("cyl", 3)])
def test_slab_residual_equals_single_grid(kind, ws):
    import torch.multiprocessing as mp
    from broadcast_gb300.partition import ColumnSlabs
    from oracle import oracle as O
    with tempfile.TemporaryDirectory() as d:
        mp.spawn(_worker_residual, args=(ws, _port(), kind, d), nprocs=ws, join=True)
        c = _case(kind)
        g = c["grid"]
        ref = O.residual(g, c["phys"], c["w"])
        slabs = ColumnSlabs(g["im"], g["jm"], ws, periodic=(kind == "cyl"))
        full = np.zeros_like(ref)
        for r in range(ws):
            z = np.load(os.path.join(d, "r%d.npz" % r))
            slabs.insert_owned(z["r"], full, r)
            norm = z["norm"]
        assert np.array_equal(H.interior(full), H.interior(ref))
        assert np.allclose(norm, np.sqrt((H.interior(ref) ** 2).sum(axis=(0, 1))), rtol=1e-14, atol=0)


def _worker_failure(rank, ws, port, mode, outdir):
    from broadcast_gb300.partition import ColumnSlabs, HaloExchange, HaloTimeout
    dist = _init(rank, ws, port, timeout=6)
    slabs = ColumnSlabs(24, 10, ws)
    w = np.zeros((slabs.local_im(rank) + 6, 16, 5), order="F")
    halo = HaloExchange(slabs, rank, timeout=2.0)
    if rank == 1:
        if mode == "exit":
            os._exit(0)  # leaves between steps, nothing in flight
        time.sleep(5.0)  # alive, never sends
        os._exit(0)
    t0 = time.time()
    try:
        halo.exchange(w)
        outcome = "no error"
    except HaloTimeout as e:
        outcome = "HaloTimeout: %s" % e
    with open(os.path.join(outdir, "rank0.txt"), "w") as f:
        f.write("%s\n%.2f\n" % (outcome, time.time() - t0))
    os._exit(0)


@pytest.mark.parametrize("mode", ["exit", "silent"])
def test_missing_neighbour_raises_instead_of_hanging(mode):
    import torch.multiprocessing as mp
    with tempfile.TemporaryDirectory() as d:
        ctx = mp.spawn(_worker_failure, args=(2, _port(), mode, d), nprocs=2, join=False)
        t0 = time.time()
        while not ctx.join(timeout=1.0):
            assert time.time() - t0 < 60.0, "ranks did not finish"
        outcome, dt = open(os.path.join(d, "rank0.txt")).read().split("\n")[:2]
        assert outcome.startswith("HaloTimeout"), outcome
        assert float(dt) < 15.0


def test_column_slabs_cover_the_grid():
    from broadcast_gb300.partition import ColumnSlabs
    for im, n in ((400, 4), (257, 3), (10, 2)):
        s = ColumnSlabs(im, 10, n)
        cols = [i for r in range(n) for i in range(s.owned(r)[0], s.owned(r)[1] + 1)]
        assert cols == list(range(1, im + 1))
        sizes = [s.local_im(r) for r in range(n)]
        assert max(sizes) - min(sizes) <= 2 and min(sizes) >= 5
    with pytest.raises(ValueError):
        ColumnSlabs(9, 10, 2)
    a = np.asfortranarray(np.random.default_rng(0).standard_normal((26, 16, 5)))
    s = ColumnSlabs(20, 10, 3)
    b = np.zeros_like(a)
    b[:3], b[-3:] = a[:3], a[-3:]
    for r in range(3):
        s.insert_owned(s.extract_cells(a, r), b, r)
    assert np.array_equal(a, b)
