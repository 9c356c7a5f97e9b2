"""Test infrastructure only: call the reference's own routines (translated
from its Fortran by oracle/ref_translate.py into oracle/_ref/libref.so).

Available only where oracle/_ref/ was built from a reference checkout
(python oracle/ref_build.py); `available()` says whether it is.  Scalars are
passed by reference as in Fortran; arrays are Fortran-ordered numpy arrays.
"""
import ctypes
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "_ref", "libref.so")
SIGS = os.path.join(HERE, "_ref", "signatures.json")
_lib = None
_sigs = None


def available():
    return os.path.exists(SO) and os.path.exists(SIGS)


def _load():
    global _lib, _sigs
    if _lib is None:
        _lib = ctypes.CDLL(SO)
        _sigs = json.load(open(SIGS))
    return _lib, _sigs


def call(name, *args):
    """Call reference routine `name` with its Fortran argument list.

    Arrays must be numpy arrays of the right dtype (float64 for real,
    int32 for integer) and Fortran order; they are modified in place.
    Scalars may be Python numbers; intent(out) scalars come back in the
    returned list (one entry per argument, arrays returned as given)."""
    lib, sigs = _load()
    sig = sigs[name]
    if len(args) != len(sig):
        raise TypeError("%s takes %d arguments, got %d" % (name, len(sig), len(args)))
    cargs, keep = [], []
    for (an, typ, is_arr), a in zip(sig, args):
        if typ == "char":
            b = ctypes.create_string_buffer(a.encode() if isinstance(a, str) else a, 64)
            keep.append(b)
            cargs.append(b)
        elif is_arr:
            want = np.float64 if typ == "real" else np.int32
            if not (isinstance(a, np.ndarray) and a.dtype == want and (a.flags.f_contiguous or a.ndim <= 1)):
                raise TypeError("%s argument %s: need Fortran-ordered %s array" % (name, an, want.__name__))
            cargs.append(ctypes.c_void_p(a.ctypes.data))
            keep.append(a)
        else:
            c = ctypes.c_double(float(a)) if typ == "real" else ctypes.c_int(int(a))
            keep.append(c)
            cargs.append(ctypes.byref(c))
    getattr(lib, "ref_" + name)(*cargs)
    out = []
    for (an, typ, is_arr), k in zip(sig, keep):
        out.append(k if (is_arr or typ == "char") else k.value)
    return out
