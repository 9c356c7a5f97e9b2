"""ctypes binding of libbroadcast_gb300.so (C ABI in include/broadcast_gb300.h).

The library is the only compute path: if it cannot be loaded the import of
any broadcast_gb300 operator raises, there is no CPU fallback.
"""
import ctypes
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libbroadcast_gb300.so")

P, I, D, S, L, Z, F = "p", "i", "d", "s", "L", "z", "f"
_CT = {P: ctypes.c_void_p, I: ctypes.c_int, D: ctypes.c_double, S: ctypes.c_char_p, L: ctypes.c_longlong,
       Z: ctypes.c_size_t, F: ctypes.c_float}

# name -> argument kinds (every function returns int unless listed in _RESTYPE)
SIGNATURES = {
    "bcg_abi_version": "",
    "bcg_set_stream": P,
    "bcg_get_stream": "",
    "bcg_synchronize": "",
    "bcg_last_error_string": "",
    "bcg_residual_scratch_bytes": "iiii",
    "bcg_flux_num_dnc5_2d": "pppppppppp" + "i" + "d" * 11 + "ii",
    "bcg_flux_num_dnc5_2d_d": "pppp" + "pppppppp" + "i" + "d" * 11 + "ii",
    "bcg_flux_num_dnc5_2d_dn": "ppppi" + "pppppppp" + "i" + "d" * 11 + "ii",
    "bcg_flux_num_dnc5_nowall_2d": "pppppppppp" + "i" + "d" * 11 + "ii",
    "bcg_flux_num_dnc5_nowall_2d_d": "pppp" + "pppppppp" + "i" + "d" * 11 + "ii",
    "bcg_impli_matrix_free_2d": "ppppppp" + "ddddd" + "ii" + "ddddd" + "iii",
    "bcg_csr_band_lu_solve": "ipppLpppip",
    "bcg_band32_factor": "ippppipp",
    "bcg_band32_solve": "Lpp",
    "bcg_band32_dims": "Lp",
    "bcg_band32_destroy": "L",
    "bcg_gmres_solve": "Lipppppiidpp",
    **{"bcg_flux_num_dnc%d%s_2d" % (o, v): "pppppppppp" + "i" + "d" * 11 + "ii" for o in (3, 7, 9) for v in ("", "_nowall")},
    **{"bcg_flux_num_dnc%d%s_2d_d" % (o, v): "pppp" + "pppppppp" + "i" + "d" * 11 + "ii"
       for o in (3, 7, 9) for v in ("", "_nowall")},
    "bcg_flux_num_dnc5_2d_b": "pppp" + "pppppppp" + "i" + "d" * 11 + "ii",
    "bcg_flux_num_dnc5_2d_bn": "ppppi" + "pppppppp" + "i" + "d" * 11 + "ii",
    "bcg_flux_num_dnc5_nowall_2d_b": "pppp" + "pppppppp" + "i" + "d" * 11 + "ii",
    "bcg_bc_wall_viscous_adia_2d": "psdpiii",
    "bcg_bc_wall_viscous_adia_2d_d": "ppsdpiii",
    "bcg_bc_no_reflexion_2d": "ppsppp" + "d" + "iiii",
    "bcg_bc_no_reflexion_2d_d": "pppsppp" + "d" + "iiii",
    "bcg_bc_supandsubinlet_2d": "psppppd" + "iiii",
    "bcg_bc_supandsubinlet_2d_d": "ppsppppd" + "iiii",
    "bcg_bc_extrapolate_o2_2d": "pspiiii",
    "bcg_bc_extrapolate_o2_2d_d": "ppspiiii",
    "bcg_bc_wall_viscous_adia_2d_b": "ppsdpiii",
    "bcg_bc_no_reflexion_2d_b": "pppsppp" + "d" + "iiii",
    "bcg_bc_supandsubinlet_2d_b": "ppsppppd" + "iiii",
    "bcg_bc_extrapolate_o2_2d_b": "ppspiiii",
    "bcg_jn_match_2d_b": "pppiiiiii" + "pppiiiiii" + "pi",
    "bcg_jn_match_2d": "ppiiiiii" + "ppiiiiii" + "pi",
    "bcg_jn_match_2d_d": "pppiiiiii" + "pppiiiiii" + "pi",
    "bcg_jn_match_geom_2d": "ppiiiiii" + "ppiiiiii" + "p",
    "bcg_testvector": "piiiiii",
    "bcg_testvector_partial": "piiiiii" + "iiii",
    "bcg_computejacobianfromjv": "pppp" + "iiiiii" + "L",
    "bcg_computejacobianfromjv_relaxed": "pppp" + "iiiiii" + "Lp",
    "bcg_computejacobianfromjv_relaxed_withjn": "pppp" + "iiiiii" + "Lp",
    "bcg_computejacobianfromjv_withjn": "pppp" + "iiiiii" + "L",
    "bcg_computejacobianfromjv_relaxed_withjnandcheck": "pppp" + "iiiiii" + "Lpdi",
    "bcg_computejacobianfromdz": "pppp" + "iiiiii" + "L",
    "bcg_compute_norml2": "pppiii",
    "bcg_compute_norml2inf": "pppiii",
    "bcg_compute_maxnorm": "ppppiii",
    "bcg_computegeom_2d": "pppppppp" + "iii",
    "bcg_set_bndbl_2d": "ppp" + "iii",
    "bcg_initblfv": "d" + "pppp" + "iii",
    "bcg_fp64_peak_tflops": P,
    "bcg_jacobian_dnc5_bl_csr": "ppppp" + "i" + "d" * 11 + "ii" + "pppp" + "pipi" + "pdi" + "ppp" + "L" + "p",
    "bcg_flux_num_dnc5_2d_noalloc": "pppppppppp" + "i" + "d" * 11 + "ii",
    "bcg_coeffs_5p_dz": "ppp" + "pppppppp" + "i" + "d" * 9 + "ii",
    "bcg_coeffs_5p_dz2": "ppp" + "pppppppp" + "i" + "d" * 9 + "ii",
    "bcg_coeffs_5p_dz_dn": "pppi" + "pppppppp" + "i" + "d" * 9 + "ii",
    "bcg_coeffs_5p_dz2_dn": "pppi" + "pppppppp" + "i" + "d" * 9 + "ii",
    "bcg_jacobian_span_bl_csr": "pppppi" + "d" * 11 + "ii" + "pppp" + "pipi" + "di" + "ppppp" + "ippppLp",
    "bcg_batch_create": "ipppip",
    "bcg_batch_set_arrays": "L" + "p" * 8,
    "bcg_batch_configure": "Liii",
    "bcg_batch_configure_host": "Liii",
    "bcg_batch_run": "Li",
    "bcg_batch_run_pass": "Li",
    "bcg_batch_run_host": "Li" + "p" * 8,
    "bcg_batch_device_bytes": "Lp",
    "bcg_batch_destroy": "L",
    "bcg_csr_spanwise_beta": "i" + "ppp" * 3 + "ip" + "ppp" + "L" + "p",
    "bcg_jacobian_dnc5_cyl_csr": "ppppp" + "i" + "d" * 11 + "ii" + "pp" + "pi" + "ppppp" + "pdi" + "ppp" + "L" + "p",
    "bcg_mlp_gemm_nn": "i" + "pppppppp" + "iiiii" + "f",
    "bcg_mlp_gemm_tn": "pppiiii",
    "bcg_mlp_colsum": "piiip",
    "bcg_mlp_adam": "pipiii" + "pppppppp" + "ffff" + "p",
    "bcg_mlp_cast_weights": "piipp",
    "bcg_mlp_features": "ppipipiLiiipp",
    "bcg_mlp_sum": "pip",
    "bcg_jacobian_dz_bl_csr": "ppppp" + "i" + "d" * 9 + "ii" + "pppp" + "pipi" + "id" + "ppp" + "L" + "p",
}
_RESTYPE = {"bcg_get_stream": ctypes.c_void_p, "bcg_last_error_string": ctypes.c_char_p,
            "bcg_residual_scratch_bytes": ctypes.c_size_t}

_lock = threading.Lock()
_lib = None


class BroadcastError(RuntimeError):
    """A bcg_* entry point returned an error code."""


def load():
    """Load (building it first if needed) the CUDA library; raise if impossible."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            from . import build as _build
            _build.build()
        lib = ctypes.CDLL(LIB_PATH)
        for name, kinds in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = [_CT[k] for k in kinds]
            fn.restype = _RESTYPE.get(name, ctypes.c_int)
        _lib = lib
        return lib


def ptr(a):
    """Raw address of a numpy array or a torch tensor (host or CUDA)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    raise TypeError("expected a numpy array or a torch tensor, got %r" % type(a))


def call(name, *args):
    """Call bcg_<name>, converting arrays to pointers; raise on a non-zero code."""
    lib = load()
    fn = getattr(lib, name)
    kinds = SIGNATURES[name]
    conv = []
    for k, a in zip(kinds, args):
        if k == P:
            conv.append(ptr(a) if not isinstance(a, int) else a)
        elif k == S:
            conv.append(a.encode() if isinstance(a, str) else a)
        else:
            conv.append(a)
    rc = fn(*conv)
    if name in _RESTYPE:
        return rc
    if rc != 0:
        msg = lib.bcg_last_error_string()
        raise BroadcastError("%s returned %d: %s" % (name, rc, msg.decode() if msg else ""))
    return rc
