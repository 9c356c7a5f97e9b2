"""Synthetic workloads of the residual hot path, built the way the reference
drivers build theirs (host-side pre-processing, run once per grid).

  bl_case   : 2-D laminar flat-plate boundary layer, single-block Cartesian
              grid, x uniform (coordinates are local Reynolds numbers under the
              reference's nondimensionalisation, BROADCAST_npz.py:615-700),
              y geometrically stretched; inlet sup/sub (Ilo), extrapolation
              (Ihi), adiabatic wall (Jlo), no-reflexion far field (Jhi)
              (card_bl2d_fv_npz.py:90-94, BROADCAST_npz.py:704-731).
  cyl_case  : 2-D cylinder O-mesh, periodic in i (azimuth), wall (Jlo) and
              no-reflexion (Jhi) (cylinder.py:400-527, handleBC.py).

Grids, metrics and states are Fortran-ordered numpy arrays with gh = 3 ghost
layers, exactly the arrays the reference passes to its f2py routines.  The
metric routine is injected (`ops`) so the same construction serves the
library (its host pre-processing entry points) and the CPU oracle.
"""
import numpy as np

GH = 3
# dimensional constants of the reference cards (card_bl2d_fv_npz.py:98-110,
# card_cyl2d.py)
GAM, RGAZ, TS, CS, MUSUTH, PRANDTL, T0 = 1.4, 287.1, 273.15, 110.4, 1.716e-5, 0.72, 288.0


def sutherland(muref, ts, cs, t):
    """BROADCAST_npz.py:121-123"""
    return muref * np.sqrt(t / ts) * ((1.0 + cs / ts) / (1.0 + cs / t))


def physics(mach, mode, reynolds=None, k2=1.01, k4=1.0):
    """Nondimensional constants (BROADCAST_npz.py:556-676, cylinder.py:298-400).

    mode 'bl' : Lref = mu_inf/(rho_inf u_inf), so x is a local Reynolds number.
    mode 'cyl': Lref = D = 1, Re = rho_inf u_inf D / mu_inf = reynolds.
    """
    muinf = sutherland(MUSUTH, TS, CS, T0)
    sound = np.sqrt(GAM * RGAZ * T0)
    uinf = mach * sound
    einf = RGAZ / (GAM - 1.0) * T0 + 0.5 * uinf * uinf
    runit = 3.4e6 if mode == "bl" else float(reynolds)
    rhoinf = runit * muinf / uinf
    pinf = rhoinf * RGAZ * T0
    cp = GAM * RGAZ / (GAM - 1.0)
    cv = RGAZ / (GAM - 1.0)
    roref, vref, tref_ = rhoinf, uinf, T0
    muref_ = muinf if mode == "bl" else roref * vref * 1.0
    pref, cvref = roref * vref ** 2, vref ** 2 / tref_
    ph = dict(cp=cp / cvref, cv=cv / cvref, prandtl=PRANDTL, gam=GAM, rgaz=RGAZ / cvref, cs=CS / tref_,
              muref=MUSUTH / muref_, tref=TS / tref_, k2=k2, k4=k4)
    ph["s_suth"] = ph["cs"]
    ph["muinf"] = muinf / muref_
    ph["einf"] = einf / vref ** 2
    ph["pinf"] = pinf / pref
    ph["mach"] = mach
    ph["state"] = np.array([1.0, 1.0, 0.0, 0.0, ph["einf"]])
    return ph


def _alloc(im, jm, gh=GH):
    ni, nj = im + 2 * gh, jm + 2 * gh
    z = lambda *s: np.zeros(s, order="F")
    return dict(im=im, jm=jm, gh=gh, x0=z(ni + 1, nj + 1), y0=z(ni + 1, nj + 1), nx=z(ni + 1, nj + 1, 2),
                ny=z(ni + 1, nj + 1, 2), xc=z(ni, nj), yc=z(ni, nj), vol=z(ni, nj), volf=z(ni, nj, 2))


def _geom(g, ops):
    if ops is None:  # the library's host geometry (srcfv/geom/computegeom.F90)
        from .srcfv import f_geom
        f_geom.computegeom_2d(g["x0"], g["y0"], g["nx"], g["ny"], g["xc"], g["yc"], g["vol"], g["volf"], g["im"],
                              g["jm"], g["gh"])
        return
    ops.computegeom(g["x0"], g["y0"], g["nx"], g["ny"], g["xc"], g["yc"], g["vol"], g["volf"], g["im"], g["jm"],
                    g["gh"])


def geometric_nodes(n, first, ratio, start=0.0):
    k = np.arange(n + 1, dtype=np.float64)
    return start + first * (ratio ** k - 1.0) / (ratio - 1.0)


def bl_grid(im, jm, x_start=1.0e5, length=5.0e5, ratio=1.03, first=None, ops=None, gh=GH):
    g = _alloc(im, jm, gh)
    gh = g["gh"]
    x = np.linspace(x_start, x_start + length, im + 1)
    if first is None:
        # delta_99 ~ 5 x / sqrt(Re_x) at the inlet, 40 cells across it
        first = 5.0 * np.sqrt(x_start) / 40.0
    y = geometric_nodes(jm, first, ratio)
    g["x0"][gh:gh + im + 1, :] = x[:, None]
    g["y0"][:, gh:gh + jm + 1] = y[None, :]
    _geom(g, ops)
    return g


def bl_interfaces(im, jm, gh=GH):
    """Fortran interf(2,2) arrays {imin,jmin; imax,jmax} (BROADCAST_npz.py:704-731)."""
    f = lambda a, b, c, d: np.array([[a, b], [c, d]], dtype=np.int32)
    return dict(Ilo=f(1, 1, 1, jm), Ihi=f(im, 1, im, jm + gh), Jlo=f(1 - gh, 1, im + gh, 1), Jhi=f(1 - gh, jm, im, jm))


def bl_case(im=400, jm=150, mach=0.5, x_start=1.0e5, length=5.0e5, ratio=1.03, noise=1.0e-4, seed=0, ops=None,
            gh=GH):
    """Boundary-layer workload: polynomial Blasius state (initialisation.f90)
    plus seeded uniform noise on the interior conserved variables.  gh = 3 for
    DNC5; the driver's (order+1)//2 (BROADCAST_npz.py:501-502) for the others."""
    ph = physics(mach, "bl")
    g = bl_grid(im, jm, x_start, length, ratio, ops=ops, gh=gh)
    gh = g["gh"]
    ni, nj = im + 2 * gh, jm + 2 * gh
    w = np.zeros((ni, nj, 5), order="F")
    w[:, :, :] = ph["state"][None, None, :]
    field = np.zeros((jm, gh, 5), order="F")
    field[:, :, :] = ph["state"][None, None, :]
    wbd = np.zeros((im + gh, 5), order="F")
    ops.initblfv(ph["muinf"], g["xc"], g["yc"], w, field, im, gh, jm)
    ops.set_bndbl(w, field, wbd, im, jm, gh)
    rng = np.random.default_rng(seed)
    w[gh:gh + im, gh:gh + jm, :] += rng.uniform(-noise, noise, size=(im, jm, 5))
    return dict(kind="bl", grid=g, phys=ph, w=w, field=field, wbd=wbd, interf=bl_interfaces(im, jm, gh))


def cyl_grid(im, jm, r_in=0.5, r_out=50.0, ratio=1.05, ops=None, gh=GH):
    g = _alloc(im, jm, gh)
    gh = g["gh"]
    first = (r_out - r_in) * (ratio - 1.0) / (ratio ** jm - 1.0)
    r = geometric_nodes(jm, first, ratio, r_in)
    r[-1] = r_out
    t = np.deg2rad(180.0 - 360.0 * np.arange(im + 1) / im)  # clockwise from the upstream point
    g["x0"][gh:gh + im + 1, gh:gh + jm + 1] = r[None, :] * np.cos(t)[:, None]
    g["y0"][gh:gh + im + 1, gh:gh + jm + 1] = r[None, :] * np.sin(t)[:, None]
    _geom(g, ops)
    # periodic joins of the cell metrics and face normals (cylinder.py:481-527)
    for a in ("xc", "yc", "vol"):
        arr = g[a]
        arr[gh + im:gh + im + gh, :] = arr[gh:2 * gh, :]          # i = im+1..im+gh  <- 1..gh
        arr[0:gh, :] = arr[im:im + gh, :]                         # i = 1-gh..0      <- im-gh+1..im
    for a in ("nx", "ny"):
        arr = g[a]
        arr[gh + im + 1:gh + im + 1 + gh, :, :] = arr[gh + 1:gh + 1 + gh, :, :]  # nodes im+2..im+1+gh <- 2..1+gh
        arr[0:gh, :, :] = arr[im:im + gh, :, :]                                  # nodes 1-gh..0 <- im+1-gh..im
    vol = g["vol"]
    vf = g["volf"]
    vf[gh:gh + im + 1, gh:gh + jm + 1, 0] = 2.0 / (vol[gh:gh + im + 1, gh:gh + jm + 1] + vol[gh - 1:gh + im, gh:gh + jm + 1])
    vf[gh:gh + im + 1, gh:gh + jm + 1, 1] = 2.0 / (vol[gh:gh + im + 1, gh:gh + jm + 1] + vol[gh:gh + im + 1, gh - 1:gh + jm])
    return g


def cyl_interfaces(im, jm, gh=GH):
    """cylinder.py:400-460: wall Jlo, no-reflexion Jhi, joins Ilo/Ihi."""
    f = lambda a, b, c, d: np.array([[a, b], [c, d]], dtype=np.int32)
    jmin, jmax = 1 - gh, jm + gh
    return dict(Jlo=f(1, 1, im, 1), Jhi=f(1, jm, im, jm), Ilo=f(1, 1 - gh, 1, jm + gh), Ihi=f(im, 1 - gh, im, jm + gh),
                prr1=f(im + 1, jmin, im + gh, jmax), prd1=f(im - gh + 1, jmin, im, jmax),
                prr2=f(1 - gh, jmin, 0, jmax), prd2=f(1, jmin, gh, jmax), tr=np.array([1, 2], dtype=np.int32))


def cyl_case(im=256, jm=256, mach=0.1, reynolds=47.0, noise=1.0e-3, seed=1, r_out=50.0, ratio=1.05, ops=None,
             gh=GH):
    """Cylinder workload: uniform flow plus seeded uniform noise (k2 = 0, k4 = 1
    as card_cyl2d.py:74-75)."""
    ph = physics(mach, "cyl", reynolds=reynolds, k2=0.0, k4=1.0)
    g = cyl_grid(im, jm, r_out=r_out, ratio=ratio, ops=ops, gh=gh)
    gh = g["gh"]
    ni, nj = im + 2 * gh, jm + 2 * gh
    w = np.zeros((ni, nj, 5), order="F")
    w[:, :, :] = ph["state"][None, None, :]
    rng = np.random.default_rng(seed)
    w[gh:gh + im, gh:gh + jm, :] += rng.uniform(-noise, noise, size=(im, jm, 5))
    wbd = np.zeros((im, 5), order="F")
    wbd[:, :] = ph["state"][None, :]
    return dict(kind="cyl", grid=g, phys=ph, w=w, wbd=wbd, interf=cyl_interfaces(im, jm, gh))


def interior(a, gh=GH):
    return a[gh:-gh, gh:-gh, ...]


def uneven_bl_spec(n=64, seed=4):
    """Sizes and Mach numbers of the uneven batch of boundary layers:
    nx ~ U{200..1200}, ny ~ U{80..300}, Mach ~ U(0.3, 0.8), drawn in that
    order per grid from default_rng(seed).  Returns the list of (im, jm, mach)
    and the generator, whose next draws are the grids' tangent directions."""
    rng = np.random.default_rng(seed)
    spec = [(int(rng.integers(200, 1201)), int(rng.integers(80, 301)), float(rng.uniform(0.3, 0.8))) for _ in range(n)]
    return spec, rng


def uneven_bl_batch(n=64, seed=4, ops=None, only=None):
    """Yield (k, case, wd) for the grids of uneven_bl_spec: grid k is
    bl_case(im, jm, mach, seed=100 + k) and its direction wd is N(0, 1) on the
    interior cells (zero ghosts), drawn in grid order from the same generator.
    `only`: the grid indices to build (the others' directions are still drawn)."""
    spec, rng = uneven_bl_spec(n, seed)
    for k, (im, jm, mach) in enumerate(spec):
        d = rng.standard_normal((im, jm, 5))
        if only is not None and k not in only:
            continue
        c = bl_case(im, jm, mach=mach, seed=100 + k, ops=ops)
        wd = np.zeros_like(c["w"])
        wd[GH:GH + im, GH:GH + jm] = d
        yield k, c, wd
