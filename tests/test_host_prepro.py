"""The library's host pre-processing entry points (bcg_computegeom_2d,
bcg_jn_match_geom_2d, bcg_initblfv, bcg_set_bndbl_2d in csrc/host.cpp,
through the f_geom / f_bnd / f_init drop-in modules) against the golden
fixtures made by the reference's own routines and against the oracle, bit for
bit.  These build the grids and states of bench.py's GPU arm, so equality with
the oracle's construction also shows that both timed arms run the same inputs.
Every routine but the periodic join runs on the host, without a GPU.

Reference: srcfv/geom/computegeom.F90:3-104, borders/jn_match_geom.F90:7-68,
initialisation.f90:2-58, set_bnd.f90:1-24."""
import numpy as np
import pytest

from broadcast_gb300 import cases
from oracle import oracle as O
from tests import golden_io as G
from tests import helpers as H


class LibOps:
    """Host pre-processing through the library (the product path)."""

    @staticmethod
    def computegeom(*a):
        from broadcast_gb300.srcfv import f_geom
        f_geom.computegeom_2d(*a)

    @staticmethod
    def initblfv(muinf, xc, yc, w, field, im, gh, jm):
        from broadcast_gb300 import f_init
        f_init.initblfv(muinf, xc, yc, w, field, im, gh, jm)

    @staticmethod
    def set_bndbl(w, field, wbd, im, jm, gh):
        from broadcast_gb300 import f_init
        f_init.set_bndbl_2d(w, field, wbd, im, jm, gh)


GEOM = ("x0", "y0", "nx", "ny", "xc", "yc", "vol", "volf")
SEEDS = {"bl_14x10": 0, "bl_23x17": 3}


def _build(kind, im, jm, ops, **kw):
    return (cases.bl_case if kind == "bl" else cases.cyl_case)(im, jm, ops=ops, **kw)


@pytest.mark.parametrize("name", G.CASES)
def test_against_golden_fixtures(name):
    """Metrics, initial state, inflow field and far-field state of the small
    golden cases through the library, against the reference's outputs."""
    d = G.load(name)
    kw = {"seed": SEEDS[name]} if d["kind"] == "bl" else {"seed": 1}
    c = _build(d["kind"], d["im"], d["jm"], LibOps, **kw)
    for k in GEOM:
        a, b = c["grid"][k], d[k]
        assert np.allclose(a, b, rtol=1e-14, atol=1e-14 * np.abs(b).max()), k
    assert np.allclose(c["w"], d["w_raw"], rtol=1e-14, atol=1e-15)
    assert np.array_equal(c["wbd"], d["wbd"])
    if d["kind"] == "bl":
        assert np.array_equal(c["field"], d["field"])


@pytest.mark.parametrize("kind,im,jm,kw", [
    ("bl", 400, 150, {"seed": 0}),                       # the 400x150 boundary layer
    ("bl", 933, 294, {"seed": 108, "mach": 0.7645131938827097}),  # one grid of the uneven batch
    ("cyl", 256, 256, {"seed": 1}),                      # the 256x256 cylinder O-mesh
    ("cyl", 61, 37, {"seed": 5, "mach": 0.2, "reynolds": 120.0}),
])
def test_bit_identical_to_oracle(kind, im, jm, kw):
    a = _build(kind, im, jm, LibOps, **kw)
    b = _build(kind, im, jm, H.OracleOps, **kw)
    for k in GEOM:
        assert np.array_equal(a["grid"][k], b["grid"][k]), k
    assert np.array_equal(a["w"], b["w"])
    assert np.array_equal(a["wbd"], b["wbd"])
    if kind == "bl":
        assert np.array_equal(a["field"], b["field"])


@pytest.mark.gpu
def test_jn_match_geom_against_oracle_join():
    """bcg_jn_match_geom_2d (one scalar field, a copy kernel on the GPU) equals the oracle's join of a
    one-variable array, and the periodic metric joins of the O-mesh
    (cylinder.py:497-527) rebuilt with it equal the grid's."""
    from broadcast_gb300.srcfv import f_bnd
    im, jm, gh = 17, 11, 3
    it = cases.cyl_interfaces(im, jm, gh)
    rng = np.random.default_rng(7)
    src = np.asfortranarray(rng.standard_normal((im + 2 * gh, jm + 2 * gh)))
    for prr, prd in ((it["prr1"], it["prd2"]), (it["prr2"], it["prd1"])):
        a, b = src.copy(order="F"), np.asfortranarray(src.copy()[:, :, None])
        f_bnd.jn_match_geom_2d(a, prr, gh, gh, gh, gh, im, jm, a, prd, gh, gh, gh, gh, im, jm, it["tr"])
        O.jn_match(b, prr, (gh,) * 4, im, jm, b, prd, (gh,) * 4, im, jm, it["tr"], 1)
        assert np.array_equal(a, b[:, :, 0])
        assert not np.array_equal(a, src)
    g = cases.cyl_grid(im, jm, ops=H.OracleOps)
    for key in ("xc", "yc", "vol"):
        x = g[key].copy(order="F")
        x[:gh, :] = 0.0
        x[im + gh:, :] = 0.0
        f_bnd.jn_match_geom_2d(x, it["prr1"], gh, gh, gh, gh, im, jm, x, it["prd2"], gh, gh, gh, gh, im, jm, it["tr"])
        f_bnd.jn_match_geom_2d(x, it["prr2"], gh, gh, gh, gh, im, jm, x, it["prd1"], gh, gh, gh, gh, im, jm, it["tr"])
        assert np.array_equal(x, g[key]), key


@pytest.mark.parametrize("im,jm", [(14, 8), (15, 10)])
@pytest.mark.parametrize("build", ["library", "oracle"])
def test_omesh_metrics_against_the_reference_driver(im, jm, build):
    """The O-mesh metrics with their periodic joins (cases.cyl_grid, through
    the library's host routines or the oracle) against the reference driver's
    own statements (cylinder.py:478-525: computegeom_2d, jn_match_geom_2d on
    xc, yc, vol, jn_match_2d on the face normals, volf), executed on the same
    nodes by tests/golden/make_omesh.py: bit for bit, ghosts included."""
    import os
    fix = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "omesh_metrics.npz"))
    g = cases.cyl_grid(im, jm, ops=None if build == "library" else H.OracleOps)
    for k in ("nx", "ny", "xc", "yc", "vol", "volf"):
        assert np.array_equal(g[k], fix["%s_%dx%d" % (k, im, jm)]), k
