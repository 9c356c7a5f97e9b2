"""Properties of the discretisation that pin the oracle beyond the golden
fixtures (CPU only).  Each property is checked on the oracle, which the CUDA
kernels match to rounding in the GPU parity tests.

- Freestream preservation of flux_num_dnc5_2d (srcfv/rhs/flux_num_dnc5.F90:7-226).
- Invariance of the O-mesh residual under a move of the branch cut (the
  periodic joins of cylinder.py:481-527 and jn_match.F90:3-66).
- The reference's own finite-difference recipe for the tangent
  (BROADCAST_npz.py:1091-1125), executed against the linearised boundary chain
  plus the tangent of flux_num_dnc5_2d_d.
- The colored 245-seed Jacobian and Dz / Dzz assemblies (misc/ComputeJacobian.f90:292-1204,
  the loops of BROADCAST_npz.py:1068-1137, 1221-1249 and cylinder.py:889-960)
  against the dense operators built column by column from unit directions.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from broadcast_gb300 import cases
from oracle import oracle as O
from tests import helpers as H


def _uniform(c, ph):
    w = np.zeros_like(c["w"], order="F")
    w[:, :, :] = ph["state"][None, None, :]
    return w


# ---- freestream preservation ----------------------------------------------------
def test_freestream_preservation():
    """A uniform state (ghosts included) on a closed-metric grid.

    Rectilinear boundary layer: the residual is exactly zero on every row of
    the interior formula (j >= 4; rows 1-3 hold the wall face and the
    off-centred rows, which do not preserve a uniform flow along a no-slip
    wall), and on every row without the wall rows, for DNC3/5/7/9.  The face
    normals repeat exactly along each grid line, so the zero is exact and does
    not depend on the platform's libm.

    Curvilinear O-mesh: the inviscid operator (mu = 0) leaves only rounding.
    The reference's viscous face gradients do not close on curvilinear cells,
    so with viscosity a uniform state leaves the metric closure error of the
    4th-order face-gradient formula (6.9e-5 of the flux scale at 21 x 14, in
    rho E through the heat flux); the translated reference gives the same
    value bit for bit, so this is the scheme's property, recorded here."""
    c = H.bl_case(20, 16, seed=1)
    g, ph = c["grid"], c["phys"]
    w = _uniform(c, ph)
    ri = H.interior(O.residual(g, ph, w))
    assert np.all(ri[:, 3:, :] == 0.0)
    assert np.all(H.interior(O.residual(g, ph, w, nowall=True)) == 0.0)
    c5 = H.bl_case(20, 16, seed=1, gh=5)
    w5 = _uniform(c5, c5["phys"])
    for order in (3, 5, 7, 9):
        r = O.residual(c5["grid"], c5["phys"], w5, order=order, nowall=True)
        assert np.all(H.interior(r, gh=5) == 0.0), order

    c = H.cyl_case(21, 14, seed=1)
    g = c["grid"]
    inviscid = dict(c["phys"], muref=0.0)
    w = _uniform(c, inviscid)
    scale = H.flux_scale(c, w).max()
    for nowall in (False, True):
        ri = H.interior(O.residual(g, inviscid, w, nowall=nowall))
        assert np.abs(ri[:, 3:, :]).max() <= 1e-14 * scale
    viscous = H.interior(O.residual(g, c["phys"], w))[:, 3:, :]
    print("O-mesh 21x14, viscous freestream residual (rows >= 4): %.2e of the flux scale"
          % (np.abs(viscous).max() / scale))


# ---- O-mesh branch cut ------------------------------------------------------------
def _cut_moved(im, jm, s, seed=1):
    """The same O-mesh and state with the branch cut moved by s cells: node
    column k of the new grid is node column (k + s) mod im of the original (the
    closing column im is column s), the state and far-field state relabeled the
    same way, the metrics and joins rebuilt as the driver builds them."""
    gh = cases.GH
    c = H.cyl_case(im, jm, seed=seed)
    x_int = c["grid"]["x0"][gh:gh + im + 1, gh:gh + jm + 1].copy()
    y_int = c["grid"]["y0"][gh:gh + im + 1, gh:gh + jm + 1].copy()
    lab = (np.arange(im + 1) + s) % im

    class Moved(H.OracleOps):
        @staticmethod
        def computegeom(x0, y0, *rest):
            x0[gh:gh + im + 1, gh:gh + jm + 1] = x_int[lab]
            y0[gh:gh + im + 1, gh:gh + jm + 1] = y_int[lab]
            O.computegeom(x0, y0, *rest)

    c2 = cases.cyl_case(im, jm, seed=seed, ops=Moved)
    cells = (np.arange(im) + s) % im
    c2["w"][gh:gh + im, gh:gh + jm] = c["w"][gh:gh + im, gh:gh + jm][cells]
    c2["wbd"] = np.asfortranarray(c["wbd"][cells])
    return c, c2, cells


@pytest.mark.parametrize("s", [1, 8])
def test_omesh_residual_under_a_moved_branch_cut(s):
    """The residual on the relabeled grid is the relabeled residual.

    The inviscid operator is invariant everywhere (rounding of the closing node
    column: sin(pi) against sin(-pi)).  With viscosity two cell columns are
    not: the last cell before the old cut and the last before the new one.
    Their viscous fluxes read the j-face normals of ghost node column im+1,
    which the driver's joins leave as computegeom's linear extrapolation (they
    join node columns im+2..im+1+gh and 1-gh..0, cylinder.py:513-521), so
    those columns depend on where the cut is.  Every other cell is invariant."""
    im, jm = 21, 14
    c, c2, cells = _cut_moved(im, jm, s)
    for phys, exempt in ((dict(c["phys"], muref=0.0), ()), (c["phys"], (im - 1, (im - 1 - s) % im))):
        w, w2 = c["w"].copy(order="F"), c2["w"].copy(order="F")
        H.oracle_bcs(c, w)
        H.oracle_bcs(c2, w2)
        r = H.interior(O.residual(c["grid"], phys, w))[cells]
        r2 = H.interior(O.residual(c2["grid"], phys, w2))
        err = (np.abs(r2 - r) / H.flux_scale(c, w).max()).max(axis=(1, 2))
        keep = np.ones(im, bool)
        keep[list(exempt)] = False
        assert err[keep].max() <= 1e-13, (s, np.nonzero(err > 1e-13)[0])
        if exempt:
            print("cut moved by %d: seam columns (new labels) %s, %.1e of the flux scale"
                  % (s, sorted(exempt), err[~keep].max()))


# ---- the reference's finite-difference recipe -----------------------------------------
EPS = 1e-6  # the recipe's epsilon at order 2 (BROADCAST_npz.py:1092)


def _recipe_residual(c, w, wd, s):
    """w + s wd with the ghosts zeroed, the drivers' boundary fills, residual."""
    gh = c["grid"]["gh"]
    w2 = w + s * wd
    w2[:gh] = 0.0
    w2[:, :gh] = 0.0
    w2[-gh:] = 0.0
    w2[:, -gh:] = 0.0
    w2 = np.asfortranarray(w2)
    H.oracle_bcs(c, w2)
    return H.interior(O.residual(c["grid"], c["phys"], w2))


@pytest.mark.parametrize("kind", ["bl", "cyl"])
def test_tangent_against_the_reference_fd_recipe(kind):
    """Every colour seed: testvector, the linearised boundary chain and the
    tangent, against the recipe's differences with epsilon 1e-6, relative to
    max|R'v| of the seed.  Where R is smooth within +-epsilon the tangent
    equals the central difference (observed within 8e-8).  Where a
    +-epsilon perturbation crosses a branch switch (the sign switches of
    bc_no_reflexion near the far field, the wall rows) R has a kink: the
    central difference is the mean of the two branches' slopes, and the
    tangent is the slope of the branch taken at w (Tapenade's convention), so
    it equals the one-sided difference on that side (observed within 9e-8).
    Every cell must match one of the two within 1e-6.  The kink cells (central
    difference off by more than 1e-6) must come from rho v seeds, in the two
    wall rows (|v| falls to ~5e-6 there, so a 1e-6 change of rho v flips the
    sign of the j-face normal velocity inside |X| of the spectral radius) or
    the three rows next to the far field (bc_no_reflexion's switches)."""
    c = H.bl_case(20, 16, seed=1) if kind == "bl" else H.cyl_case(21, 14, seed=1)
    g, ph = c["grid"], c["phys"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    w = c["w"].copy(order="F")
    H.oracle_bcs(c, w)
    r0 = _recipe_residual(c, w, np.zeros_like(w), 0.0)
    kinks, kink_seeds, worst = 0, set(), 0.0
    for m in range(5):
        for l in range(7):
            for k in range(7):
                wd = O.testvector(m, l, k, gh, im, jm)
                H.oracle_bcs(c, w.copy(order="F"), wd)
                _, rd = O.jvp(g, ph, w, wd)
                t = H.interior(rd)
                rp, rm = _recipe_residual(c, w, wd, EPS), _recipe_residual(c, w, wd, -EPS)
                scale = np.abs(t).max()
                central = np.abs(t - (rp - rm) / (2 * EPS)) / scale
                side = np.minimum(np.abs(t - (rp - r0) / EPS), np.abs(t - (r0 - rm) / EPS)) / scale
                kink = central > 1e-6
                assert np.all(side[kink] <= 1e-6), ((m, l, k), central.max(), side[kink].max())
                if kink.any():
                    rows = np.nonzero(kink)[1] + 1
                    assert m == 2 and np.all((rows <= 2) | (rows >= jm - 2)), ((m, l, k), sorted(set(rows)))
                    kinks += int(kink.sum())
                    kink_seeds.add((m, l, k))
                worst = max(worst, central[~kink].max())
    print("%s: cells within 1e-6 of the central difference (worst %.1e); %d kink cells in seeds %s"
          % (kind, worst, kinks, sorted(kink_seeds)))
    if kind == "cyl":
        assert kinks == 0


# ---- colored assembly against dense columns ------------------------------------------
def _dense_jacobian(c, w):
    """-dR/dw column by column: a unit direction on each interior (i, j, v),
    the linearised boundary chain, the tangent; rows and columns in the
    assembly's order e + 5 j + 5 jm i (0-based)."""
    g, ph = c["grid"], c["phys"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    n = 5 * im * jm
    D = np.zeros((n, n))
    for i in range(im):
        for j in range(jm):
            wds = []
            for v in range(5):
                wd = np.zeros_like(w, order="F")
                wd[i + gh, j + gh, v] = 1.0
                H.oracle_bcs(c, w.copy(order="F"), wd)
                wds.append(wd)
            _, rds = O.jvp(g, ph, w, np.stack(wds))
            for v in range(5):
                D[:, v + 5 * j + 5 * jm * i] = -H.interior(rds[v]).reshape(-1)
    return D


@pytest.mark.parametrize("kind", ["bl", "cyl_withjn", "cyl_zones"])
def test_colored_assembly_equals_dense_columns(kind):
    """The colored assembly (245 seeds of distance-7 colouring; on an O-mesh
    whose im is not a multiple of 7, the driver's two azimuthal zones with
    testvector_partial and computejacobianfromjv_relaxed_withjnandcheck) is the
    dense Jacobian bit for bit: every dependency of the residual, boundary
    fills and periodic joins included, lies within the colouring's reach."""
    c = {"bl": lambda: H.bl_case(14, 14, seed=1), "cyl_withjn": lambda: H.cyl_case(14, 12, seed=1),
         "cyl_zones": lambda: H.cyl_case(15, 12, seed=1)}[kind]()
    g, ph = c["grid"], c["phys"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    w = c["w"].copy(order="F")
    H.oracle_bcs(c, w)
    n, nb = 5 * im * jm, im * jm * 49 * 25
    mini = 2e-16
    seeds = [(m, l, k) for m in range(5) for l in range(7) for k in range(7)]
    if kind == "cyl_zones":
        jac, ia, ja = np.zeros(2 * nb), np.zeros(2 * nb, np.int32), np.zeros(2 * nb, np.int32)
        imid = im // 2 // 7 * 7
        cd = np.zeros((im, jm), order="F")
        for zn, (i0, i1) in enumerate([(0, imid - 1), (imid, im - 1)]):
            for (m, l, k) in seeds:
                wd = O.testvector_partial(m, l, k, gh, im, jm, i0, i1, 0, jm - 1)
                H.oracle_bcs(c, w.copy(order="F"), wd)
                _, rd = O.jvp(g, ph, w, wd)
                O.computejacobian_withjnandcheck(jac, ia, ja, rd, m, l, k, gh, im, jm, cd, mini, zn)
    else:
        mode = O.JAC_PLAIN if kind == "bl" else O.JAC_WITHJN
        jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
        for (m, l, k) in seeds:
            wd = O.testvector(m, l, k, gh, im, jm)
            H.oracle_bcs(c, w.copy(order="F"), wd)
            _, rd = O.jvp(g, ph, w, wd)
            O.computejacobian(mode, jac, ia, ja, rd, m, l, k, gh, im, jm, None)
    keep = (ia >= 0) & (ia < n) & (np.abs(jac) > mini)
    A = sp.csr_matrix((jac[keep], (ia[keep], ja[keep])), shape=(n, n)).toarray()
    D = _dense_jacobian(c, w)
    D[np.abs(D) <= mini] = 0.0
    assert np.array_equal(A, D), np.abs(A - D).max()


@pytest.mark.parametrize("which", ["dz", "dzz"])
def test_spanwise_assembly_equals_dense_columns(which):
    """The Dz / Dzz assembly of BROADCAST_npz.py:1221-1249 (testvector, the
    linearised boundary chain, coeffs_5p_dz / coeffs_5p_dz2,
    computejacobianfromdz, the 2e-16 filter) is the dense operator built from
    unit columns bit for bit."""
    op = O.dz if which == "dz" else O.dzz
    c = H.bl_case(14, 14, seed=1)
    g, ph = c["grid"], c["phys"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    w = c["w"].copy(order="F")
    H.oracle_bcs(c, w)
    n, nb, mini = 5 * im * jm, im * jm * 49 * 25, 2e-16
    jac, ia, ja = np.zeros(nb), np.zeros(nb, np.int32), np.zeros(nb, np.int32)
    for m in range(5):
        for l in range(7):
            for k in range(7):
                wd = O.testvector(m, l, k, gh, im, jm)
                H.oracle_bcs(c, w.copy(order="F"), wd)
                O.computejacobian(O.JAC_DZ, jac, ia, ja, op(g, ph, w, wd), m, l, k, gh, im, jm, None)
    keep = (ia >= 0) & (ia < n) & (np.abs(jac) > mini)
    A = sp.csr_matrix((jac[keep], (ia[keep], ja[keep])), shape=(n, n)).toarray()
    D = np.zeros((n, n))
    for i in range(im):
        for j in range(jm):
            wds = []
            for v in range(5):
                wd = np.zeros_like(w, order="F")
                wd[i + gh, j + gh, v] = 1.0
                H.oracle_bcs(c, w.copy(order="F"), wd)
                wds.append(wd)
            out = op(g, ph, w, np.stack(wds))
            for v in range(5):
                D[:, v + 5 * j + 5 * jm * i] = H.interior(out[v]).reshape(-1)
    D[np.abs(D) <= mini] = 0.0
    assert np.array_equal(A, D), np.abs(A - D).max()


# ---- adjoint dot-product identity through the boundary chain -----------------------
def test_adjoint_chain_dot_product():
    """<T x, u> = <x, T^T u> for T = (interior of) the residual tangent after
    the boundary-layer chain of tangent fills (inlet, no-reflexion,
    extrapolation, wall; BROADCAST_npz.py:1079-1085), and T^T = the residual
    adjoint (flux_num_dnc5_b.f90) followed by the fill adjoints in reverse
    order (bc_*_b.f90), with x and u random on the interior; to 1e-12."""
    c = H.bl_case(24, 18, seed=2)
    g, ph, it = c["grid"], c["phys"], c["interf"]
    im, jm, gh = g["im"], g["jm"], g["gh"]
    w = c["w"].copy(order="F")
    H.oracle_bcs(c, w)
    rng = np.random.default_rng(31)
    x = np.zeros_like(w, order="F")
    x[gh:-gh, gh:-gh] = rng.standard_normal((im, jm, 5))
    u = np.zeros_like(w, order="F")
    u[gh:-gh, gh:-gh] = rng.standard_normal((im, jm, 5))
    steps = [("inlet", "Ilo"), ("noref", "Jhi"), ("extrap", "Ihi"), ("wall", "Jlo")]
    states, ws, tx = [], w.copy(order="F"), x.copy(order="F")
    for kind, loc in steps:
        states.append(ws.copy(order="F"))
        if kind == "inlet":
            O.bc_inlet(ws, loc, it[loc], c["field"], g["nx"], g["ny"], ph["gam"], im, jm, gh, wd=tx)
        elif kind == "noref":
            O.bc_noref(ws, c["wbd"], loc, it[loc], g["nx"], g["ny"], ph["gam"], gh, im, jm, wd=tx)
        elif kind == "extrap":
            O.bc_extrap(ws, loc, it[loc], im, jm, gh, wd=tx)
        else:
            O.bc_wall(ws, loc, ph["gam"], it[loc], gh, im, jm, wd=tx)
    _, jx = O.jvp(g, ph, ws, tx)
    lhs = float(np.sum(H.interior(jx) * H.interior(u)))
    wb = O.vjp(g, ph, ws, u)
    for (kind, loc), st in zip(reversed(steps), reversed(states)):
        aux = {"inlet": c["field"], "noref": c["wbd"]}.get(kind)
        O.bc_adjoint(kind, st, wb, loc, it[loc], gh, im, jm, gam=ph["gam"], aux=aux, nx=g["nx"], ny=g["ny"])
    rhs = float(np.sum(x * wb))
    scale = float(np.sum(np.abs(H.interior(jx) * H.interior(u))))
    assert abs(lhs - rhs) <= 1e-12 * scale, (lhs, rhs)
