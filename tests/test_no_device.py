"""Without a GPU nothing computes: every compute entry point of the library
returns an error code, and the drop-in modules raise.  This is the C-ABI side
of "no CPU fallback": the only routines that succeed on a machine without a
CUDA device are the host pre-processing of csrc/host.cpp (computegeom_2d,
initblfv, set_bndbl_2d, which the reference also runs once per grid on the
host) and the bookkeeping calls.  Runs where no CUDA device is visible; each
export is called in a child process with dummy buffers.
"""
import os
import subprocess
import sys
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HOST_ROUTINES = {"bcg_computegeom_2d", "bcg_initblfv", "bcg_set_bndbl_2d"}
BOOKKEEPING = {"bcg_abi_version", "bcg_set_stream", "bcg_get_stream", "bcg_last_error_string",
               "bcg_residual_scratch_bytes"}

CHILD = textwrap.dedent(r"""
    import json, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    from broadcast_gb300 import _lib
    L = _lib.load()
    buf = np.zeros(1 << 20)
    out = {}
    for name, kinds in _lib.SIGNATURES.items():
        args = [buf.ctypes.data if k == "p" else b"Ilo" if k == "s" else 1.0 if k in "df" else 8 for k in kinds]
        rc = getattr(L, name)(*args)
        out[name] = rc if isinstance(rc, int) else None
    print(json.dumps(out))
""")


def _device_visible():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_device_visible(), reason="a CUDA device is visible")
def test_every_compute_entry_point_fails_without_a_device():
    import json
    p = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, (p.returncode, p.stderr[-2000:])
    rc = json.loads(p.stdout.strip().splitlines()[-1])
    for name in HOST_ROUTINES:
        assert rc[name] == 0, name
    compute = {n: v for n, v in rc.items() if n not in HOST_ROUTINES | BOOKKEEPING}
    assert len(compute) >= 80
    bad = {n: v for n, v in compute.items() if v not in (-4, -1)}
    assert not bad, bad
    assert sum(v == -4 for v in compute.values()) >= 60


@pytest.mark.skipif(_device_visible(), reason="a CUDA device is visible")
def test_drop_in_module_raises_without_a_device():
    import numpy as np
    from broadcast_gb300._lib import BroadcastError
    from broadcast_gb300.srcfv import f_sch
    from tests import helpers as H
    c = H.bl_case(20, 16, seed=1)
    g, ph = c["grid"], c["phys"]
    res = np.zeros_like(c["w"], order="F")
    with pytest.raises(BroadcastError, match="-4"):
        f_sch.flux_num_dnc5_2d(res, c["w"], g["x0"], g["y0"], g["nx"], g["ny"], g["xc"], g["yc"], g["vol"],
                               g["volf"], 3, *[ph[k] for k in ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref",
                                                                "tref", "s_suth", "k2", "k4")])
    assert not res.any()
