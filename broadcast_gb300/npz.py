"""The NPZ "tree" files through which the reference's drivers hand a base flow
and its Jacobian lists to the stability scripts (BROADCAST_npz.py:247-333,
407-467; read by biglobal.py:40-61 and resolvent_all.py), with the same keys,
so files written here are read unchanged downstream and vice versa.

writeNPZ / readNPZtree / fillNPZ / fillNPZ_3D keep the reference's names and
argument order.  The Jacobian lists (IA, JA, Aij) are COO triplets: the
reference stores them in seed-slot order after remove_zero_jac, the CSR
assembled on the GPU gives them row by row (csr_to_lists); downstream
createMatPetscCSR (misc/PETSc_func.py:71-96) sorts them into the same CSR
either way.
"""
import numpy as np

STATE_KEYS = ("x0", "y0", "xc", "yc", "vol", "volf", "nx", "ny", "im", "jm", "gh", "FlowSolutionInit",
              "ResidualInit", "interf1", "interf2", "interf3", "interf4", "BC1", "BC2", "BC3", "BC4", "Wbd", "Field",
              "SchemeType", "Scheme", "k2", "k4", "Mach", "Prandtl", "Rgaz", "Cp", "Cv", "Gamma",
              "TemperatureSutherland", "TemperatureRefSutherland", "ViscosityRefSutherland", "Pref", "CFL",
              "Freqres", "Freqsort")


def _path(filename):
    return filename + ".npz"


def writeNPZ(filename, im, jm, gh, w, x0, y0, vol, volf, nx, ny, xc, yc, field, wbd, res, sch, k2, k4, interf1,
             interf2, interf3, interf4, lf, cp, cv, gam, cs, tref, muref, rgaz, mach, prandtl, cfl, freqres, freqsort,
             pinf=None):
    """BROADCAST_npz.py:247-262: state, metrics, boundary set-up and constants.
    lf = [routinein, routineout, routinenr, routinew, routinesch, libbnd, libsch]."""
    routinein, routineout, routinenr, routinew, routinesch, libbnd, libsch = lf[:7]
    np.savez(_path(filename), x0=x0, y0=y0, xc=xc, yc=yc, vol=vol, volf=volf, nx=nx, ny=ny, im=im, jm=jm, gh=gh,
             FlowSolutionInit=np.array(w, copy=True), ResidualInit=np.array(res, copy=True), interf1=interf1,
             interf2=interf2, interf3=interf3, interf4=interf4, BC1=libbnd + "." + routinein,
             BC2=libbnd + "." + routineout, BC3=libbnd + "." + routinew, BC4=libbnd + "." + routinenr, Wbd=wbd,
             Field=field, SchemeType=sch, Scheme=libsch + "." + routinesch, k2=k2, k4=k4, Mach=mach, Prandtl=prandtl,
             Rgaz=rgaz, Cp=cp, Cv=cv, Gamma=gam, TemperatureSutherland=cs, TemperatureRefSutherland=tref,
             ViscosityRefSutherland=muref, Pref=pinf, CFL=cfl, Freqres=freqres, Freqsort=freqsort)


def _s(a):
    return np.array2string(a)[1:-1]


def readNPZtree(filename):
    """BROADCAST_npz.py:407-467: the same 36-tuple, EndOfRun state when present."""
    dic = np.load(_path(filename), allow_pickle=True)
    if "FlowSolutionEndOfRun" in dic:
        w, res = dic["FlowSolutionEndOfRun"], dic["ResidualEndOfRun"]
    else:
        w, res = dic["FlowSolutionInit"], dic["ResidualInit"]
    libsch, routinesch = _s(dic["Scheme"]).split(".")
    libbnd, routinein = _s(dic["BC1"]).split(".")
    _, routineout = _s(dic["BC2"]).split(".")
    _, routinew = _s(dic["BC3"]).split(".")
    _, routinenr = _s(dic["BC4"]).split(".")
    lf = [routinein, routineout, routinenr, routinew, routinesch, libbnd, libsch]
    return (dic["im"], dic["jm"], dic["gh"], w, dic["x0"], dic["y0"], dic["vol"], dic["volf"], dic["nx"], dic["ny"],
            dic["xc"], dic["yc"], dic["Field"], dic["Wbd"], res, _s(dic["SchemeType"]), dic["k2"], dic["k4"],
            dic["interf1"], dic["interf2"], dic["interf3"], dic["interf4"], lf, dic["Cp"], dic["Cv"], dic["Gamma"],
            dic["TemperatureSutherland"], dic["TemperatureRefSutherland"], dic["ViscosityRefSutherland"],
            dic["Rgaz"], dic["Mach"], dic["Prandtl"], dic["Pref"], dic["CFL"], dic["Freqres"], dic["Freqsort"])


def fillNPZ(filename, w, res, IA, JA, Jacvol, gh):
    """BROADCAST_npz.py:311-320: add the end-of-run state and the Jacobian lists."""
    dic = dict(np.load(_path(filename), allow_pickle=True))
    dic.update(ResidualEndOfRun=res, FlowSolutionEndOfRun=w, IA=IA, JA=JA, Aij=Jacvol)
    np.savez(_path(filename), **dic)


def fillNPZ_3D(filename, IAdz, JAdz, Jacdz, IAdz2, JAdz2, Jacdz2):
    """BROADCAST_npz.py:323-333: add the Dz and Dzz lists."""
    dic = dict(np.load(_path(filename), allow_pickle=True))
    dic.update(IAdz=IAdz, JAdz=JAdz, Aijdz=Jacdz, IAdz2=IAdz2, JAdz2=JAdz2, Aijdz2=Jacdz2)
    np.savez(_path(filename), **dic)


def csr_to_lists(indptr, indices, data):
    """CSR (host numpy or torch arrays) -> the (IA, JA, Aij) lists of the NPZ file."""
    to_np = lambda a: a.detach().cpu().numpy() if hasattr(a, "detach") else np.asarray(a)
    indptr, indices, data = to_np(indptr), to_np(indices), to_np(data)
    nnz = int(indptr[-1])
    ia = np.repeat(np.arange(len(indptr) - 1, dtype=np.int32), np.diff(indptr).astype(np.int64))
    return ia, np.ascontiguousarray(indices[:nnz], dtype=np.int32), np.ascontiguousarray(data[:nnz], dtype=np.float64)
