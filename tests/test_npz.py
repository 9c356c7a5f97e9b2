"""NPZ tree files (broadcast_gb300.npz) with the reference's keys and calls
(BROADCAST_npz.py:247-333, 407-467), and CSR -> (IA, JA, Aij) lists that
rebuild the same matrix as the reference's COO lists."""
import numpy as np
import pytest

from broadcast_gb300 import npz
from tests import helpers as H


def _write(tmp_path, c):
    g, ph, it = c["grid"], c["phys"], c["interf"]
    lf = ["bc_supandsubinlet_2d", "bc_extrapolate_o2_2d", "bc_no_reflexion_2d", "bc_wall_viscous_adia_2d",
          "flux_num_dnc5_2d", "f_bnd", "f_sch"]
    fn = str(tmp_path / "bl")
    res = np.zeros_like(c["w"])
    npz.writeNPZ(fn, g["im"], g["jm"], g["gh"], c["w"], g["x0"], g["y0"], g["vol"], g["volf"], g["nx"], g["ny"],
                 g["xc"], g["yc"], c["field"], c["wbd"], res, "dnc5", ph["k2"], ph["k4"], it["Ilo"], it["Ihi"],
                 it["Jlo"], it["Jhi"], lf, ph["cp"], ph["cv"], ph["gam"], ph["cs"], ph["tref"], ph["muref"],
                 ph["rgaz"], 0.5, ph["prandtl"], 1.0, 10, 100, pinf=1.0)
    return fn, lf


def test_write_read_round_trip(tmp_path):
    c = H.bl_case(14, 10)
    fn, lf = _write(tmp_path, c)
    keys = set(np.load(fn + ".npz", allow_pickle=True).files)
    assert keys == set(npz.STATE_KEYS)
    t = npz.readNPZtree(fn)
    assert len(t) == 36
    assert int(t[0]) == 14 and int(t[1]) == 10 and int(t[2]) == 3
    assert np.array_equal(t[3], c["w"]) and np.array_equal(t[8], c["grid"]["nx"])
    assert t[15] == "dnc5" and t[22] == lf
    w2 = c["w"] * 2.0
    ia, ja, a = np.array([0, 1], np.int32), np.array([1, 0], np.int32), np.array([1.5, -2.0])
    npz.fillNPZ(fn, w2, np.ones_like(w2), ia, ja, a, 3)
    npz.fillNPZ_3D(fn, ia, ja, a, ia, ja, 2 * a)
    d = np.load(fn + ".npz", allow_pickle=True)
    for k in ("FlowSolutionEndOfRun", "ResidualEndOfRun", "IA", "JA", "Aij", "IAdz", "JAdz", "Aijdz", "IAdz2",
              "JAdz2", "Aijdz2"):
        assert k in d.files
    assert np.array_equal(npz.readNPZtree(fn)[3], w2)  # EndOfRun state preferred


def test_lists_from_csr_rebuild_the_matrix():
    sp = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(0)
    a = sp.random(50, 50, density=0.1, random_state=1, format="csr")
    a.sort_indices()
    ia, ja, v = npz.csr_to_lists(a.indptr, a.indices, a.data)
    perm = rng.permutation(len(v))  # the reference's lists come in seed-slot order
    b = sp.csr_matrix((v[perm], (ia[perm], ja[perm])), shape=a.shape)  # createMatPetscCSR's conversion
    assert (a != b).nnz == 0


def _reference_inputs():
    """The inputs tests/golden/make_npz.py gave the reference's writer."""
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "make_npz.py")
    spec = importlib.util.spec_from_file_location("make_npz", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.inputs(), mod.OUT


def test_reads_the_file_the_reference_writes():
    """tests/golden/npz_tree_bl_10x8.npz was written by the reference's own
    writeNPZ, fillNPZ and fillNPZ_3D (BROADCAST_npz.py:247-333); readNPZtree
    returns what they were given, the end-of-run state and residual first."""
    (args, fill, _), fn = _reference_inputs()
    t = npz.readNPZtree(fn)
    assert len(t) == 36
    assert (int(t[0]), int(t[1]), int(t[2])) == args[:3]
    assert np.array_equal(t[3], fill[0]) and np.array_equal(t[14], fill[1])
    for q in range(4, 14):
        assert np.array_equal(t[q], args[q]), q
    assert t[15] == "dnc5" and t[22] == args[22]
    for q in (18, 19, 20, 21):
        assert np.array_equal(t[q], args[q]), q


def test_writes_what_the_reference_writes(tmp_path):
    """The same calls through this package give the same file: the same keys,
    and under each key the same dtype, shape, memory order and values."""
    (args, fill, fill3), ref_fn = _reference_inputs()
    fn = str(tmp_path / "tree")
    npz.writeNPZ(fn, *args, pinf=1.0)
    npz.fillNPZ(fn, *fill)
    npz.fillNPZ_3D(fn, *fill3)
    mine, ref = np.load(fn + ".npz"), np.load(ref_fn + ".npz")
    assert set(mine.files) == set(ref.files)
    for k in ref.files:
        a, b = mine[k], ref[k]
        assert a.dtype == b.dtype and a.shape == b.shape, k
        assert a.flags.f_contiguous == b.flags.f_contiguous and a.flags.c_contiguous == b.flags.c_contiguous, k
        assert np.array_equal(a, b), k
