"""The host-array JVP path with many directions (bcg_flux_num_dnc5_2d_dn with
numpy inputs): uploads, residual passes and downloads run pipelined in up to
four chunks of whole 4-direction groups on separate streams.  Results must equal the device-array path, the
ghosts of the host outputs must stay untouched, and back-to-back calls must
not see each other's buffers."""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu
PHYS = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")


def _host_call(c, wd, nd, pinned):
    import torch
    from broadcast_gb300 import _lib
    g = c["grid"]
    n = c["w"].size
    mk = (lambda k: torch.empty(k, dtype=torch.float64, pin_memory=True).numpy()) if pinned else np.empty
    wdh = mk(n * nd)
    wdh[:] = np.concatenate([np.ravel(x, order="F") for x in wd])
    res, resd = mk(n), mk(n * nd)
    res[:], resd[:] = 7.0, 7.0
    _lib.call("bcg_flux_num_dnc5_2d_dn", res, resd, c["w"], wdh, nd, None, None, g["nx"], g["ny"], None, None,
              g["vol"], g["volf"], 3, *[float(c["phys"][k]) for k in PHYS], g["im"], g["jm"])
    return res.reshape(c["w"].shape, order="F"), [resd[k * n:(k + 1) * n].reshape(c["w"].shape, order="F")
                                                   for k in range(nd)]


@pytest.mark.parametrize("nd,pinned", [(8, True), (13, True), (20, True), (32, False)])
def test_pipelined_host_path_equals_device_path(nd, pinned):
    from broadcast_gb300.operator import Dnc5Operator, to_device, to_host
    import torch
    c = H.cyl_case(64, 40)
    H.oracle_bcs(c, c["w"])
    rng = np.random.default_rng(nd)
    wd = [np.asfortranarray(rng.standard_normal(c["w"].shape)) for _ in range(nd)]
    op = Dnc5Operator(c["grid"], c["phys"])
    r_dev, rd_dev = op.jvp(to_device(c["w"]), torch.stack([to_device(x) for x in wd]))
    res, resd = _host_call(c, wd, nd, pinned)
    ghost = np.ones(c["w"].shape, bool)
    ghost[3:-3, 3:-3] = False
    assert np.all(res[ghost] == 7.0)
    assert H.rel_err(res, to_host(r_dev), H.flux_scale(c, c["w"])) < 1e-13
    for k in range(nd):
        ref = to_host(rd_dev[k])
        sc = np.abs(H.interior(ref)).reshape(-1, 5).max(0)
        assert H.rel_err(resd[k], ref, sc) < 1e-13
        assert np.all(resd[k][ghost] == 7.0)
    # a second call right after, with other directions, through the same pool buffers
    wd2 = [x * -0.5 for x in wd]
    _, resd2 = _host_call(c, wd2, nd, pinned)
    for k in range(nd):
        ref = to_host(rd_dev[k]) * -0.5
        sc = np.abs(H.interior(ref)).reshape(-1, 5).max(0)
        assert H.rel_err(resd2[k], ref, sc) < 1e-12
