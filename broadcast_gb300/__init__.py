"""GB300 (sm_103a) implementation of BROADCAST's DNC5 residual / tangent /
boundary-condition / colored-Jacobian hot path.

  broadcast_gb300.srcfv.f_sch, f_lin, f_adj, f_bnd, f_dz, f_norm, f_geom, broadcast_gb300.misc.f_misc,
  broadcast_gb300.f_init : f2py-compatible drop-ins for the reference modules
  broadcast_gb300.operator : device-resident operator API (torch CUDA tensors)
  broadcast_gb300.autograd : the residual as a torch.autograd.Function (tangent / adjoint kernels)
  broadcast_gb300.cases    : synthetic workloads built like the reference drivers'

All compute runs in libbroadcast_gb300.so (include/broadcast_gb300.h).
"""
from ._lib import BroadcastError, load  # noqa: F401

__all__ = ["BroadcastError", "load"]
