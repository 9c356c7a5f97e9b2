"""The library's residual and tangent kernels on column slabs
(broadcast_gb300.partition) reproduce the single-grid GPU results on the owned
columns, for the open boundary-layer grid and the periodic O-mesh (one
process, slabs evaluated one after another; the multi-rank exchange itself
is covered on CPU ranks in test_partition.py)."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,n", [("bl", 3), ("cyl", 4)])
def test_slabs_match_full_grid_on_gpu(kind, n):
    from broadcast_gb300.operator import Dnc5Operator, to_device, to_host
    from broadcast_gb300.partition import ColumnSlabs
    c = H.bl_case(61, 24) if kind == "bl" else H.cyl_case(64, 20)
    H.oracle_bcs(c, c["w"])
    g = c["grid"]
    rng = np.random.default_rng(4)
    wd = np.zeros_like(c["w"])
    wd[3:-3, 3:-3] = rng.standard_normal((g["im"], g["jm"], 5))
    H.oracle_bcs(c, c["w"].copy(order="F"), wd)  # ghosts of the direction from the linearised chain
    op = Dnc5Operator(g, c["phys"])
    res, resd = op.jvp(to_device(c["w"]), to_device(wd))
    ref, refd = to_host(res), to_host(resd)
    slabs = ColumnSlabs(g["im"], g["jm"], n, periodic=(kind == "cyl"))
    full, fulld = np.zeros_like(ref), np.zeros_like(ref)
    for r in range(n):
        lop = Dnc5Operator(slabs.extract_grid(g, r), c["phys"])
        lr, lrd = lop.jvp(to_device(slabs.extract_cells(c["w"], r)), to_device(slabs.extract_cells(wd, r)))
        slabs.insert_owned(to_host(lr), full, r)
        slabs.insert_owned(to_host(lrd), fulld, r)
    assert np.array_equal(H.interior(full), H.interior(ref))
    assert np.array_equal(H.interior(fulld), H.interior(refd))
