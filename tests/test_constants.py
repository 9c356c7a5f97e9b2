"""The nondimensional constants of broadcast_gb300.cases.physics against the
ones the reference's drivers compute (BROADCAST_npz.py:555-669 for the
boundary layer, cylinder.py:298-400 for the cylinder), stored in
tests/golden/constants.json by tests/golden/make_constants.py, which executes
the drivers' own statements on the cards' physical constants (CPU only).

Every constant is bit-identical.
"""
import json
import os

import numpy as np
import pytest

from broadcast_gb300 import cases

FIX = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "constants.json")))
KEYS = ("gam", "cp", "cv", "rgaz", "prandtl", "cs", "muref", "tref", "muinf", "einf", "pinf")


def _compare(ph, ref):
    for k in KEYS:
        assert ph[k] == ref[k], (k, ph[k], ref[k])
    assert np.array_equal(ph["state"], ref["state"])
    assert ph["s_suth"] == ph["cs"]  # the drivers pass cs for s_suth (BROADCAST_npz.py:1031)


@pytest.mark.parametrize("entry", FIX["bl"], ids=lambda e: "M%g" % e["mach"])
def test_boundary_layer_constants(entry):
    assert entry["runit"] == 3.4e6  # the unit Reynolds number of card_bl2d_fv_npz.py
    _compare(cases.physics(entry["mach"], "bl"), entry["constants"])


@pytest.mark.parametrize("entry", FIX["cyl"], ids=lambda e: "M%g-Re%g" % (e["mach"], e["reynolds"]))
def test_cylinder_constants(entry):
    _compare(cases.physics(entry["mach"], "cyl", reynolds=entry["reynolds"]), entry["constants"])
