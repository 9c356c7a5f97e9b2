"""Argument handling shared by the f2py-compatible operator modules.

The reference calls its Fortran through f2py: arrays are Fortran-ordered
float64 numpy arrays modified in place, trailing dimension arguments are
optional and inferred from array shapes, intent(out) results are returned.
Here the same calls also accept torch CUDA tensors laid out in Fortran order
(strides (1, n0, n0*n1, ...)), which the library uses in place on the device.
"""
import numpy as np

from . import _lib


def is_torch(a):
    return hasattr(a, "data_ptr") and hasattr(a, "is_cuda")


def fortran_ok(a):
    if isinstance(a, np.ndarray):
        return a.dtype == np.float64 and a.flags.f_contiguous
    if is_torch(a):
        import torch
        if a.dtype != torch.float64:
            return False
        exp, s = [], 1
        for n in a.shape:
            exp.append(s)
            s *= n
        return all(st == e or n == 1 for st, e, n in zip(a.stride(), exp, a.shape))
    return False


def arr(a, name, inout=False):
    """Validate an array argument; inputs that are not Fortran-ordered float64
    numpy arrays are converted (like f2py), in-place ones must already be."""
    if is_torch(a):
        if not fortran_ok(a):
            raise ValueError("%s: torch tensor must be float64 with Fortran (column-major) strides" % name)
        return a
    if isinstance(a, np.ndarray) and fortran_ok(a):
        return a
    if inout:
        raise ValueError("%s: in-place argument must be a Fortran-ordered float64 array" % name)
    return np.asfortranarray(a, dtype=np.float64)


def shape(a):
    return tuple(a.shape)


def interf4(interf):
    """Fortran (2,2) integer array (given as a numpy (2,2) array in the
    reference's convention interf[0] = (imin, jmin), interf[1] = (imax, jmax),
    float or int) -> column-major int32 {imin, imax, jmin, jmax}."""
    a = np.asarray(interf)
    if is_torch(interf):
        a = interf.detach().cpu().numpy()
    a = np.asarray(np.rint(a), dtype=np.int32).reshape(2, 2)
    return np.ascontiguousarray(a.T.ravel())


def dims_from_cell(a, gh):
    n0, n1 = shape(a)[:2]
    return n0 - 2 * gh, n1 - 2 * gh


def call(name, *args):
    return _lib.call(name, *args)
