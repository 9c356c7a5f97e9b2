"""The allocation-free residual entry point (bcg_flux_num_dnc5_2d_noalloc).

It exists for callers that cannot have the library allocate device memory
during a call (a framework whose allocator already owns the GPU's memory, a
fixed memory budget, loops that cannot absorb cudaMalloc's synchronisation).
Its scratch is a fixed static device array shared by every call, so the test
checks two calls in a row against the regular entry point -- with a changed
state, and after a call on another grid, so that an entry of the shared
scratch read before this call wrote it would show -- plus the two rejections
it documents (too large a grid, host arrays).  This file is named to be
collected last.
"""
import numpy as np
import pytest

from tests import helpers as H

pytestmark = pytest.mark.gpu

PHYS = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")


def _dev_case(kind, im, jm):
    from broadcast_gb300.operator import to_device
    c = H.bl_case(im, jm) if kind == "bl" else H.cyl_case(im, jm)
    H.oracle_bcs(c, c["w"])
    g = c["grid"]
    d = {k: to_device(g[k]) for k in ("nx", "ny", "vol", "volf")}
    d["w"] = to_device(c["w"])
    return c, d


def _call(name, c, d, res):
    from broadcast_gb300 import _lib
    g, ph = c["grid"], c["phys"]
    _lib.call(name, res, d["w"], None, None, d["nx"], d["ny"], None, None, d["vol"], d["volf"], g["gh"],
              *[float(ph[k]) for k in PHYS], g["im"], g["jm"])


@pytest.mark.parametrize("kind,im,jm", [("bl", 40, 30), ("cyl", 256, 256)])
def test_noalloc_matches_regular_entry_point_twice(kind, im, jm):
    import torch
    from broadcast_gb300 import _lib
    from broadcast_gb300.operator import to_host
    _lib.load()
    _lib.call("bcg_set_stream", torch.cuda.current_stream().cuda_stream)
    c, d = _dev_case(kind, im, jm)
    ref = torch.zeros_like(d["w"])
    _call("bcg_flux_num_dnc5_2d", c, d, ref)
    scale = H.flux_scale(c, c["w"])
    for _ in range(2):  # two calls in a row on the shared static scratch
        out = torch.full_like(d["w"], 3.0)
        _call("bcg_flux_num_dnc5_2d_noalloc", c, d, out)
        torch.cuda.synchronize()
        assert H.rel_err(to_host(out), to_host(ref), scale) < 1e-12
        assert bool((out[:, :3, :] == 3.0).all())  # ghosts untouched


def test_noalloc_rejects_oversized_grid_and_host_arrays():
    import torch
    from broadcast_gb300 import _lib
    c, d = _dev_case("cyl", 28, 20)
    g, ph = c["grid"], c["phys"]
    out = torch.zeros_like(d["w"])
    # a 600 x 600 grid needs more than the fixed scratch: refused before any
    # array is touched
    with pytest.raises(_lib.BroadcastError, match="too large"):
        _lib.call("bcg_flux_num_dnc5_2d_noalloc", out, d["w"], None, None, d["nx"], d["ny"], None, None, d["vol"],
                  d["volf"], 3, *[float(ph[k]) for k in PHYS], 600, 600)
    with pytest.raises(_lib.BroadcastError, match="device pointer"):
        _call("bcg_flux_num_dnc5_2d_noalloc", c, {**d, "w": c["w"]}, out)


def test_noalloc_after_a_different_grid_and_state():
    """A 256 x 256 cylinder call fills the shared scratch with its own values;
    the 40 x 30 boundary layer after it, and again with its interior state
    scaled, must each equal the regular entry point on the same state."""
    import torch
    from broadcast_gb300 import _lib
    from broadcast_gb300.operator import to_host
    _lib.load()
    _lib.call("bcg_set_stream", torch.cuda.current_stream().cuda_stream)
    cc, dc = _dev_case("cyl", 256, 256)
    _call("bcg_flux_num_dnc5_2d_noalloc", cc, dc, torch.zeros_like(dc["w"]))
    c, d = _dev_case("bl", 40, 30)
    for scale in (1.0, 1.0005):
        w = d["w"].clone()
        w[:, 3:-3, 3:-3] *= scale
        dd = {**d, "w": w}
        ref = torch.zeros_like(w)
        _call("bcg_flux_num_dnc5_2d", c, dd, ref)
        out = torch.zeros_like(w)
        _call("bcg_flux_num_dnc5_2d_noalloc", c, dd, out)
        torch.cuda.synchronize()
        assert H.rel_err(to_host(out), to_host(ref), H.flux_scale(c, c["w"])) < 1e-12
