"""Device-resident operator API over libbroadcast_gb300.so.

States live on the GPU as torch float64 tensors whose memory is the
reference's Fortran layout: a padded state (ni, nj, 5) in Fortran order is a
C-contiguous tensor of shape (5, nj, ni); a stack of K tangent states is
(K, 5, nj, ni).  Calls are asynchronous on the library stream, which is
bound to torch's current CUDA stream at construction.
"""
import numpy as np

from . import _lib
from .cases import GH


def to_device(a, device="cuda"):
    """Fortran-ordered numpy array -> C-contiguous torch tensor, reversed shape."""
    import torch
    a = np.asfortranarray(a, dtype=np.float64)
    t = torch.from_numpy(np.ravel(a, order="F").copy()).view(*reversed(a.shape))
    return t.to(device)


def to_host(t, shape=None):
    """Inverse of to_device (shape: the Fortran shape)."""
    a = t.detach().cpu().numpy()
    shp = tuple(reversed(a.shape)) if shape is None else shape
    return np.reshape(np.ravel(a), shp, order="F")


class Dnc5Operator:
    """Residual R(w) and its tangent/adjoint on one grid, geometry resident."""

    PHYS_KEYS = ("cp", "cv", "prandtl", "gam", "rgaz", "cs", "muref", "tref", "s_suth", "k2", "k4")

    def __init__(self, grid, phys, device="cuda"):
        import torch
        _lib.load()
        self.im, self.jm, self.gh = int(grid["im"]), int(grid["jm"]), int(grid["gh"])
        if self.gh != GH:
            raise ValueError("DNC5 needs gh = 3")
        self.ni, self.nj = self.im + 2 * self.gh, self.jm + 2 * self.gh
        self.device = device
        self.nx = to_device(grid["nx"], device)
        self.ny = to_device(grid["ny"], device)
        self.vol = to_device(grid["vol"], device)
        self.volf = to_device(grid["volf"], device)
        self.phys = [float(phys[k]) for k in self.PHYS_KEYS]
        self.stream = torch.cuda.current_stream(torch.device(device))
        _lib.call("bcg_set_stream", self.stream.cuda_stream)

    @property
    def state_shape(self):
        return (5, self.nj, self.ni)

    def new_state(self, k=None):
        import torch
        shp = self.state_shape if k is None else (k,) + self.state_shape
        return torch.zeros(shp, dtype=torch.float64, device=self.device)

    def residual(self, w, res=None):
        res = self.new_state() if res is None else res
        _lib.call("bcg_flux_num_dnc5_2d", res, w, None, None, self.nx, self.ny, None, None, self.vol, self.volf,
                  self.gh, *self.phys, self.im, self.jm)
        return res

    def jvp(self, w, wd, res=None, resd=None):
        """Residual and K directional derivatives: wd is (K, 5, nj, ni) or (5, nj, ni)."""
        single = wd.dim() == 3
        wds = wd.unsqueeze(0) if single else wd
        res = self.new_state() if res is None else res
        resd = self.new_state(wds.shape[0]) if resd is None else resd
        _lib.call("bcg_flux_num_dnc5_2d_dn", res, resd, w, wds.contiguous(), wds.shape[0], None, None, self.nx,
                  self.ny, None, None, self.vol, self.volf, self.gh, *self.phys, self.im, self.jm)
        return res, (resd[0] if single else resd)

    def vjp(self, w, rb, wb=None):
        """wb = (dR/dw)^T rb over every padded cell; rb is one interior
        cotangent (5, nj, ni) or K of them (K, 5, nj, ni), all K in one call;
        rb is left unchanged here (the library consumes a copy)."""
        if rb.dim() == 4:
            k = rb.shape[0]
            wb = self.new_state(k) if wb is None else wb
            rbc = rb.detach().clone().contiguous()
            _lib.call("bcg_flux_num_dnc5_2d_bn", None, rbc, w, wb, k, None, None, self.nx, self.ny, None, None,
                      self.vol, self.volf, self.gh, *self.phys, self.im, self.jm)
            return wb
        wb = self.new_state() if wb is None else wb
        rbc = rb.detach().clone().contiguous()
        _lib.call("bcg_flux_num_dnc5_2d_b", None, rbc, w, wb, None, None, self.nx, self.ny, None, None, self.vol,
                  self.volf, self.gh, *self.phys, self.im, self.jm)
        return wb
