"""torch.autograd front end of the DNC5 residual.

`residual(w, op)` returns R(w) (interior written, ghost entries zero) for a
ghost-filled state w of shape (5, nj, ni) (Fortran layout, see
broadcast_gb300.operator) and differentiates through the library's kernels:

  reverse mode (torch.autograd.grad, .backward): the adjoint kernels,
      wb = (dR/dw)^T rb  (srcfv/adjoint/flux_num_dnc5_b.f90);
  forward mode (torch.autograd.forward_ad, torch.func.jvp): the fused
      residual + tangent kernels, R'(w) wd  (srcfv/tangent/flux_num_dnc5_d.f90).

The derivative is taken with respect to every padded cell of w, ghosts
included; the boundary fills that produce the ghosts are separate steps.
"""
import torch


class ResidualFunction(torch.autograd.Function):
    """R(w) with the library's tangent (jvp) and adjoint (backward)."""

    @staticmethod
    def forward(w, op):
        return op.residual(w.detach().contiguous())

    @staticmethod
    def setup_context(ctx, inputs, output):
        w, op = inputs
        ctx.op = op
        ctx.save_for_backward(w)
        ctx.save_for_forward(w)

    @staticmethod
    def backward(ctx, grad):
        (w,) = ctx.saved_tensors
        return ctx.op.vjp(w.detach().contiguous(), grad.contiguous()), None

    @staticmethod
    def jvp(ctx, w_t, _op_t):
        (w,) = ctx.saved_tensors
        _, resd = ctx.op.jvp(w.detach().contiguous(), w_t.contiguous())
        return resd


def residual(w, op):
    """R(w) on the GPU, differentiable in forward and reverse mode."""
    return ResidualFunction.apply(w, op)
