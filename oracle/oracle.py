"""Test infrastructure only: ctypes front end of the CPU oracle (liboracle.so).

The oracle is a C++ restatement of the reference Fortran (broadcast_oracle.hpp),
used as the checker by tests/, __graft_entry__.smoke() and the cpu_baseline
leg of bench.py.  The shipped library never calls it.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
LIB_OMP = os.path.join(BUILD, "liboracle_omp.so")
SOURCES = [os.path.join(HERE, f) for f in ("oracle_capi.cpp", "broadcast_oracle.hpp", "dual.hpp")]

_P, _I, _D, _S, _L = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_char_p, ctypes.c_longlong
_PHYS = [_D] * 11
SIGS = {
    "orc_flux_num_dnc5_2d": [_P] * 6 + [_I] + _PHYS + [_I, _I],
    "orc_flux_num_dnc5_2d_d": [_P] * 4 + [_I] + [_P] * 4 + [_I] + _PHYS + [_I, _I],
    "orc_flux_num_dnc5_2d_b": [_P] * 3 + [_P] * 4 + [_I] + _PHYS + [_I, _I],
    "orc_flux_num_dnc5_nowall_2d_b": [_P] * 3 + [_P] * 4 + [_I] + _PHYS + [_I, _I],
    "orc_flux_num_dnc5_nowall_2d": [_P] * 6 + [_I] + _PHYS + [_I, _I],
    "orc_flux_num_dnc5_nowall_2d_d": [_P] * 4 + [_I] + [_P] * 4 + [_I] + _PHYS + [_I, _I],
    "orc_flux_num_dnc5_2d_opcount": [_P] * 6 + [_I] + _PHYS + [_I, _I],
    "orc_flux_num_dnc_2d": [_I, _I] + [_P] * 6 + [_I] + _PHYS + [_I, _I],
    "orc_impli_matrix_free_2d": [_P] * 7 + [_D] * 5 + [_I, _I] + [_D] * 5 + [_I, _I],
    "orc_flux_num_dnc_2d_d": [_I, _I] + [_P] * 4 + [_I] + [_P] * 4 + [_I] + _PHYS + [_I, _I],
    "orc_bc_wall_viscous_adia_2d": [_P, _S, _D, _P, _I, _I, _I],
    "orc_bc_wall_viscous_adia_2d_d": [_P, _P, _S, _D, _P, _I, _I, _I],
    "orc_bc_no_reflexion_2d": [_P, _P, _I, _S, _P, _P, _P, _D, _I, _I, _I],
    "orc_bc_no_reflexion_2d_d": [_P, _P, _P, _I, _S, _P, _P, _P, _D, _I, _I, _I],
    "orc_bc_supandsubinlet_2d": [_P, _S, _P, _P, _I, _P, _P, _D, _I, _I, _I],
    "orc_bc_supandsubinlet_2d_d": [_P, _P, _S, _P, _P, _I, _P, _P, _D, _I, _I, _I],
    "orc_bc_extrapolate_o2_2d": [_P, _S, _P, _I, _I, _I, _I],
    "orc_bc_extrapolate_o2_2d_d": [_P, _P, _S, _P, _I, _I, _I, _I],
    "orc_jn_match_2d": [_P, _P] + [_I] * 6 + [_P, _P] + [_I] * 6 + [_P, _I],
    "orc_computegeom_2d": [_P] * 8 + [_I] * 3,
    "orc_compute_norml2": [_P] * 3 + [_I] * 3,
    "orc_compute_norml2inf": [_P] * 3 + [_I] * 3,
    "orc_compute_maxnorm": [_P] * 4 + [_I] * 3,
    "orc_initblfv": [_D] + [_P] * 4 + [_I] * 3,
    "orc_set_bndbl_2d": [_P] * 3 + [_I] * 3,
    "orc_testvector": [_P] + [_I] * 6,
    "orc_testvector_partial": [_P] + [_I] * 10,
    "orc_computejacobian": [_I, _P, _P, _P, _P] + [_I] * 6 + [_P],
    "orc_computejacobian_withjnandcheck": [_P, _P, _P, _P] + [_I] * 6 + [_P, _D, _I],
    "orc_computejacobian_band": [_I, _P, _P, _P, _P] + [_I] * 6 + [_P, _I, _I],
    "orc_coeffs_5p_dz": [_P] * 3 + [_I] + [_P] * 3 + [_I] + [_D] * 9 + [_I] * 3,
    "orc_bc_b": [_I, _P, _P, _P, _I, _S, _P, _P, _P, _D, _I, _I, _I, _I],
}

_lock = threading.Lock()
_libs = {}


def build(openmp=False, force=False):
    """Compile the oracle (strict IEEE evaluation order, no FMA contraction)."""
    os.makedirs(BUILD, exist_ok=True)
    out = LIB_OMP if openmp else LIB
    stale = force or not os.path.exists(out) or any(os.path.getmtime(s) > os.path.getmtime(out) for s in SOURCES)
    if stale:
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", out,
               os.path.join(HERE, "oracle_capi.cpp")]
        if openmp:
            cmd.insert(1, "-fopenmp")
        subprocess.run(cmd, check=True)
    return out


def lib(openmp=False):
    with _lock:
        key = bool(openmp)
        if key not in _libs:
            path = build(openmp=openmp)
            l = ctypes.CDLL(path)
            for name, at in SIGS.items():
                f = getattr(l, name)
                f.argtypes = at
                f.restype = _L if name.endswith("opcount") else _I
            _libs[key] = l
        return _libs[key]


def _p(a):
    return None if a is None else a.ctypes.data


def _phys(ph):
    return [ph[k] for k in ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")]


def _chk(a):
    assert isinstance(a, np.ndarray) and a.flags.f_contiguous and a.dtype == np.float64, "F-ordered float64 array expected"
    return a


# ---- residual -----------------------------------------------------------------
def residual(grid, ph, w, nowall=False, order=5):
    """flux_num_dnc{order}_2d, or flux_num_dnc{order}_nowall_2d with nowall=True
    (order 3, 5, 7 or 9)."""
    res = np.zeros_like(w, order="F")
    args = (_p(res), _p(_chk(w)), _p(grid["nx"]), _p(grid["ny"]), _p(grid["vol"]), _p(grid["volf"]), grid["gh"],
            *_phys(ph), grid["im"], grid["jm"])
    if order != 5:
        if lib().orc_flux_num_dnc_2d(order, 0 if nowall else 1, *args):
            raise ValueError("flux_num_dnc%d_2d: bad order or ghost width" % order)
        return res
    fn = lib().orc_flux_num_dnc5_nowall_2d if nowall else lib().orc_flux_num_dnc5_2d
    fn(*args)
    return res


def jvp(grid, ph, w, wd, nowall=False, order=5, openmp=False):
    """wd: one padded state or a stack (nd, ...) of them; returns (res, resd).
    openmp: the OpenMP build (all host cores over j-rows)."""
    wd = np.asarray(wd)
    single = wd.ndim == 3
    wds = wd[None] if single else wd
    nd = wds.shape[0]
    flat = np.stack([np.asfortranarray(x) for x in wds])
    buf = np.concatenate([np.ravel(x, order="F") for x in flat])
    out = np.zeros_like(buf)
    res = np.zeros_like(w, order="F")
    args = (_p(res), _p(out), _p(_chk(w)), _p(buf), nd, _p(grid["nx"]), _p(grid["ny"]), _p(grid["vol"]),
            _p(grid["volf"]), grid["gh"], *_phys(ph), grid["im"], grid["jm"])
    L = lib(openmp=openmp)
    if order != 5:
        if L.orc_flux_num_dnc_2d_d(order, 0 if nowall else 1, *args):
            raise ValueError("flux_num_dnc%d_2d_d: bad order or ghost width" % order)
    else:
        fn = L.orc_flux_num_dnc5_nowall_2d_d if nowall else L.orc_flux_num_dnc5_2d_d
        fn(*args)
    n = w.size
    resd = [np.reshape(out[k * n:(k + 1) * n], w.shape, order="F") for k in range(nd)]
    return res, (resd[0] if single else np.stack(resd))


def impli_matrix_free(grid, ph, w, dw, dtcoef, cfl, lmax):
    """impli_matrix_free_2d: the increment dwi for right-hand side dw (the
    driver passes the residual), lmax Gauss-Seidel sweeps; s_suth = cs as the
    drivers call it."""
    dwi = np.zeros_like(w, order="F")
    lib().orc_impli_matrix_free_2d(_p(dwi), _p(grid["nx"]), _p(grid["ny"]), _p(_chk(w)), _p(_chk(dw)),
                                   _p(grid["vol"]), _p(grid["volf"]), dtcoef, cfl, ph["gam"], ph["rgaz"],
                                   ph["prandtl"], lmax, grid["gh"], ph["cv"], ph["cs"], ph["muref"], ph["tref"],
                                   ph["cs"], grid["im"], grid["jm"])
    return dwi


def vjp(grid, ph, w, rb, nowall=False):
    """wb = (dR/dw)^T rb over all padded cells (rb interior only); nowall: the
    scheme without the wall rows."""
    rb = np.array(rb, order="F", copy=True)
    wb = np.zeros_like(w, order="F")
    (lib().orc_flux_num_dnc5_nowall_2d_b if nowall else lib().orc_flux_num_dnc5_2d_b)(_p(rb), _p(_chk(w)), _p(wb), _p(grid["nx"]), _p(grid["ny"]), _p(grid["vol"]),
                                 _p(grid["volf"]), grid["gh"], *_phys(ph), grid["im"], grid["jm"])
    return wb


def _span(which, grid, ph, w, wd, out):
    wd = np.asarray(wd)
    single = wd.ndim == 3
    wds = wd[None] if single else wd
    nd = wds.shape[0]
    buf = np.concatenate([np.ravel(np.asfortranarray(x), order="F") for x in wds])
    if out is None:
        ob = np.zeros_like(buf)
    else:
        outs = out[None] if single else out
        ob = np.concatenate([np.ravel(np.asfortranarray(x), order="F") for x in outs])
    keys = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth")
    lib().orc_coeffs_5p_dz(_p(ob), _p(_chk(w)), _p(buf), nd, _p(grid["nx"]), _p(grid["ny"]), _p(grid["vol"]),
                           grid["gh"], *[float(ph[k]) for k in keys], grid["im"], grid["jm"], which)
    n = w.size
    r = [np.reshape(ob[k * n:(k + 1) * n], w.shape, order="F") for k in range(nd)]
    return r[0] if single else np.stack(r)


def dz(grid, ph, w, wd, out=None):
    """coeffs_5p_dz: the Dz operator applied to wd (one padded state or a stack);
    ghosts of `out` (zeros if None) are kept."""
    return _span(1, grid, ph, w, wd, out)


def dzz(grid, ph, w, wd, out=None):
    """coeffs_5p_dz2: the Dzz operator applied to wd."""
    return _span(2, grid, ph, w, wd, out)


OP_KINDS = ("add_aa", "add_ap", "mul_aa", "mul_ap", "div_aa", "div_ap", "div_pa", "sqrt", "tanh", "abs", "max", "pow")
# extra flops per tangent direction for each primal operation kind (dual.hpp
# rules: d(a*b) = da*b + a*db, d(a/b) = (da - (a/b) db)/b, ...)
TANGENT_COST = dict(add_aa=1, add_ap=0, mul_aa=3, mul_ap=1, div_aa=3, div_ap=1, div_pa=2, sqrt=2, tanh=3, abs=0, max=0,
                    pow=3)


def opcount(grid, ph, w):
    """Operation tallies of one residual evaluation -> (primal flops, tangent
    flops per direction, tallies dict)."""
    counts = np.zeros(len(OP_KINDS), dtype=np.int64)
    lib().orc_flux_num_dnc5_2d_opcount(_p(counts), _p(_chk(w)), _p(grid["nx"]), _p(grid["ny"]), _p(grid["vol"]),
                                       _p(grid["volf"]), grid["gh"], *_phys(ph), grid["im"], grid["jm"])
    t = dict(zip(OP_KINDS, (int(x) for x in counts)))
    primal = sum(t.values())
    tangent = sum(TANGENT_COST[k] * v for k, v in t.items())
    return primal, tangent, t


# ---- boundary conditions -----------------------------------------------------------
def _i4(interf):
    a = np.asarray(interf, dtype=np.int32)
    return np.ascontiguousarray(a.reshape(2, 2).T.ravel()) if a.shape == (2, 2) else np.ascontiguousarray(a)


def bc_wall(w, loc, gam, interf, gh, im, jm, wd=None):
    it = _i4(interf)
    if wd is None:
        lib().orc_bc_wall_viscous_adia_2d(_p(w), loc.encode(), gam, _p(it), gh, im, jm)
    else:
        lib().orc_bc_wall_viscous_adia_2d_d(_p(w), _p(wd), loc.encode(), gam, _p(it), gh, im, jm)


def bc_noref(w, wbd, loc, interf, nx, ny, gam, gh, im, jm, wd=None):
    it = _i4(interf)
    lm = wbd.shape[0]
    if wd is None:
        lib().orc_bc_no_reflexion_2d(_p(w), _p(wbd), lm, loc.encode(), _p(it), _p(nx), _p(ny), gam, gh, im, jm)
    else:
        lib().orc_bc_no_reflexion_2d_d(_p(w), _p(wd), _p(wbd), lm, loc.encode(), _p(it), _p(nx), _p(ny), gam, gh,
                                       im, jm)


def bc_inlet(w, loc, interf, field, nx, ny, gam, im, jm, gh, wd=None):
    it = _i4(interf)
    lm = field.shape[0]
    if wd is None:
        lib().orc_bc_supandsubinlet_2d(_p(w), loc.encode(), _p(it), _p(field), lm, _p(nx), _p(ny), gam, im, jm, gh)
    else:
        lib().orc_bc_supandsubinlet_2d_d(_p(w), _p(wd), loc.encode(), _p(it), _p(field), lm, _p(nx), _p(ny), gam,
                                         im, jm, gh)


def bc_extrap(w, loc, interf, im, jm, gh, wd=None):
    it = _i4(interf)
    em = w.shape[2] if w.ndim == 3 else 1
    if wd is None:
        lib().orc_bc_extrapolate_o2_2d(_p(w), loc.encode(), _p(it), im, jm, gh, em)
    else:
        lib().orc_bc_extrapolate_o2_2d_d(_p(w), _p(wd), loc.encode(), _p(it), im, jm, gh, em)


BC_KIND = {"wall": 0, "noref": 1, "inlet": 2, "extrap": 3}


def bc_adjoint(kind, w, wb, loc, interf, gh, im, jm, gam=1.4, aux=None, nx=None, ny=None, em=5):
    """Transpose of a ghost fill (adjoint/bc_*_b.f90): wb updated in place."""
    lm = 0 if aux is None else aux.shape[0]
    lib().orc_bc_b(BC_KIND[kind], _p(_chk(w)), _p(_chk(wb)), None if aux is None else _p(aux), lm, loc.encode(),
                   _p(_i4(interf)), None if nx is None else _p(nx), None if ny is None else _p(ny), float(gam), gh, im,
                   jm, em)
    return wb


def jn_match(wr, prr, ghr, imr, jmr, wd, prd, ghd, imd, jmd, tr, em):
    a, b = _i4(prr), _i4(prd)
    t = np.ascontiguousarray(np.asarray(tr, dtype=np.int32))
    lib().orc_jn_match_2d(_p(wr), _p(a), *ghr, imr, jmr, _p(wd), _p(b), *ghd, imd, jmd, _p(t), em)


# ---- geometry, norms, seeding ------------------------------------------------------
def computegeom(x0, y0, nx, ny, xc, yc, vol, volf, im, jm, gh):
    lib().orc_computegeom_2d(_p(x0), _p(y0), _p(nx), _p(ny), _p(xc), _p(yc), _p(vol), _p(volf), im, jm, gh)


def norml2(rhs, im, jm, gh):
    a, b = np.zeros(5), np.zeros(5)
    lib().orc_compute_norml2(_p(a), _p(b), _p(rhs), im, jm, gh)
    return a, b


def norml2inf(rhs, im, jm, gh):
    a, b = np.zeros(5), np.zeros(5)
    lib().orc_compute_norml2inf(_p(a), _p(b), _p(rhs), im, jm, gh)
    return a, b


def maxnorm(rhs, im, jm, gh):
    a = np.zeros(5)
    i, j = np.zeros(5, np.int32), np.zeros(5, np.int32)
    lib().orc_compute_maxnorm(_p(a), _p(i), _p(j), _p(rhs), im, jm, gh)
    return a, i, j


def testvector(m, l, k, gh, im, jm):
    wd = np.zeros((im + 2 * gh, jm + 2 * gh, 5), order="F")
    lib().orc_testvector(_p(wd), m, l, k, gh, im, jm)
    return wd


def testvector_partial(m, l, k, gh, im, jm, istart, iend, jstart, jend):
    wd = np.zeros((im + 2 * gh, jm + 2 * gh, 5), order="F")
    lib().orc_testvector_partial(_p(wd), m, l, k, gh, im, jm, istart, iend, jstart, jend)
    return wd


JAC_PLAIN, JAC_RELAXED, JAC_RELAXED_WITHJN, JAC_WITHJN, JAC_DZ = 0, 1, 2, 3, 4


def computejacobian(mode, jac, ia, ja, resd, m, l, k, gh, im, jm, coefdiag=None):
    cd = None if coefdiag is None else np.asfortranarray(coefdiag, dtype=np.float64)
    lib().orc_computejacobian(mode, _p(jac), _p(ia), _p(ja), _p(resd), m, l, k, gh, im, jm, _p(cd))


def computejacobian_band(mode, resd, m, l, k, gh, im, jm, coefdiag=None, i0=1, i1=None):
    """The COO slots of seed (m, l, k) for the outputs of columns i0..i1
    (1-based, inclusive): (ia, ja, jac) arrays of 5 jm (i1 - i0 + 1) slots in
    the order (i, j, e) with i fastest; invalid slots carry the reference's
    marker row."""
    i1 = im if i1 is None else i1
    n = 5 * jm * (i1 - i0 + 1)
    jac, ia, ja = np.zeros(n), np.zeros(n, np.int32), np.zeros(n, np.int32)
    cd = None if coefdiag is None else np.asfortranarray(coefdiag, dtype=np.float64)
    if lib().orc_computejacobian_band(mode, _p(jac), _p(ia), _p(ja), _p(resd), m, l, k, gh, im, jm, _p(cd), i0, i1):
        raise ValueError("computejacobian_band: bad column range")
    return ia, ja, jac


def computejacobian_withjnandcheck(jac, ia, ja, resd, m, l, k, gh, im, jm, coefdiag, mini, n):
    cd = np.asfortranarray(coefdiag, dtype=np.float64)
    lib().orc_computejacobian_withjnandcheck(_p(jac), _p(ia), _p(ja), _p(resd), m, l, k, gh, im, jm, _p(cd), mini, n)


def initblfv(muinf, xc, yc, w, field, im, gh, jm):
    lib().orc_initblfv(muinf, _p(xc), _p(yc), _p(w), _p(field), im, gh, jm)


def set_bndbl(w, field, wbd, im, jm, gh):
    lib().orc_set_bndbl_2d(_p(w), _p(field), _p(wbd), im, jm, gh)
