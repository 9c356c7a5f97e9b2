"""Drop-in for the reference's misc.f_misc (misc/ComputeJacobian.f90).

testvector, testvector_partial and the COO fills of one colour seed; the
reference calls them once per seed from its Python assembly loop
(BROADCAST_npz.py:1068-1131, cylinder.py:896-981).
"""
from .._f2py import arr, call, dims_from_cell, shape


def _dims(a, gh, im, jm):
    if im is None or jm is None:
        im, jm = dims_from_cell(a, gh)
    return int(im), int(jm)


def _n(a):
    return int(shape(a)[0])


def testvector(wd, m, l, k, gh, im=None, jm=None):
    im, jm = _dims(wd, gh, im, jm)
    call("bcg_testvector", arr(wd, "wd", True), int(m), int(l), int(k), int(gh), im, jm)


def testvector_partial(wd, m, l, k, gh, im, jm, istart, iend, jstart, jend):
    call("bcg_testvector_partial", arr(wd, "wd", True), int(m), int(l), int(k), int(gh), int(im), int(jm), int(istart),
         int(iend), int(jstart), int(jend))


def computejacobianfromjv(jac, ia, ja, resd, m, l, k, gh, im=None, jm=None, nbentry=None):
    im, jm = _dims(resd, gh, im, jm)
    call("bcg_computejacobianfromjv", jac, ia, ja, arr(resd, "resd"), int(m), int(l), int(k), int(gh), im, jm,
         _n(jac) if nbentry is None else int(nbentry))


def computejacobianfromjv_relaxed(jac, ia, ja, resd, m, l, k, gh, coefdiag, im=None, jm=None, nbentry=None):
    im, jm = _dims(resd, gh, im, jm)
    call("bcg_computejacobianfromjv_relaxed", jac, ia, ja, arr(resd, "resd"), int(m), int(l), int(k), int(gh), im, jm,
         _n(jac) if nbentry is None else int(nbentry), arr(coefdiag, "coefdiag"))


def computejacobianfromjv_relaxed_withjn(jac, ia, ja, resd, m, l, k, gh, coefdiag, im=None, jm=None, nbentry=None):
    im, jm = _dims(resd, gh, im, jm)
    call("bcg_computejacobianfromjv_relaxed_withjn", jac, ia, ja, arr(resd, "resd"), int(m), int(l), int(k), int(gh),
         im, jm, _n(jac) if nbentry is None else int(nbentry), arr(coefdiag, "coefdiag"))


def computejacobianfromjv_withjn(jac, ia, ja, resd, m, l, k, gh, im=None, jm=None, nbentry=None):
    im, jm = _dims(resd, gh, im, jm)
    call("bcg_computejacobianfromjv_withjn", jac, ia, ja, arr(resd, "resd"), int(m), int(l), int(k), int(gh), im, jm,
         _n(jac) if nbentry is None else int(nbentry))


def computejacobianfromjv_relaxed_withjnandcheck(jac, ia, ja, resd, m, l, k, gh, coefdiag, mini, n, im=None, jm=None,
                                                 nbentry=None):
    im, jm = _dims(resd, gh, im, jm)
    call("bcg_computejacobianfromjv_relaxed_withjnandcheck", jac, ia, ja, arr(resd, "resd"), int(m), int(l), int(k),
         int(gh), im, jm, _n(jac) if nbentry is None else int(nbentry), arr(coefdiag, "coefdiag"), float(mini), int(n))


def computejacobianfromdz(jac, ia, ja, dz, m, l, k, gh, im=None, jm=None, nbentry=None):
    im, jm = _dims(dz, gh, im, jm)
    call("bcg_computejacobianfromdz", jac, ia, ja, arr(dz, "dz"), int(m), int(l), int(k), int(gh), im, jm,
         _n(jac) if nbentry is None else int(nbentry))
