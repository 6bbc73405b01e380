"""torch.autograd pair of the forward projector and its exact transpose.

ForwardProjection(vol) = P vol runs mct_fp; its backward is P^T (mct_fp_adjoint).
BackProjection(sgm) = P^T sgm runs mct_fp_adjoint; its backward is P (mct_fp).
The two are each other's hand-written adjoint (<P x, y> = <x, P^T y>), so losses
built from them -- data fidelity, TV, PICCS -- differentiate with torch autograd.
No counterpart in the reference (its CGLS uses an unmatched backprojector).
"""
import torch

from . import ops


class _ForwardProjection(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vol, dg, mask):
        ctx.dg = dg
        ctx.mask = mask
        return ops.fp(dg, vol.detach().contiguous(), mask=mask)

    @staticmethod
    def backward(ctx, grad):
        g = ops.fp_adjoint(ctx.dg, grad.contiguous().float(), mask=ctx.mask) if ctx.needs_input_grad[0] else None
        return g, None, None


class _BackProjection(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sgm, dg, mask):
        ctx.dg = dg
        ctx.mask = mask
        return ops.fp_adjoint(dg, sgm.detach().contiguous(), mask=mask)

    @staticmethod
    def backward(ctx, grad):
        g = ops.fp(ctx.dg, grad.contiguous().float(), mask=ctx.mask) if ctx.needs_input_grad[0] else None
        return g, None, None


def forward_project(vol, dg, mask=None):
    """Differentiable P vol: [z, y, x] -> [rows, views, cols]."""
    return _ForwardProjection.apply(vol, dg, mask)


def back_project(sgm, dg, mask=None):
    """Differentiable P^T sgm: [rows, views, cols] -> [z, y, x]."""
    return _BackProjection.apply(sgm, dg, mask)


class Projector(torch.nn.Module):
    """Module wrapper holding one forward-projector geometry (see geometry.fpj_geometry
    and geometry.ir_geometry)."""

    def __init__(self, dg, mask=None):
        super().__init__()
        self.dg = dg
        self.mask = mask

    def forward(self, vol):
        return forward_project(vol, self.dg, self.mask)

    def adjoint(self, sgm):
        return back_project(sgm, self.dg, self.mask)


def tv_isotropic(x, beta):
    """sum sqrt(|D x|^2 + beta) with the reference's forward differences
    (run_mgfbp_iterative_recon_IRN_CGLS.py:245-254), differentiable in torch."""
    gy = torch.zeros_like(x)
    gx = torch.zeros_like(x)
    gz = torch.zeros_like(x)
    gy[:, :-1, :] = x[:, 1:, :] - x[:, :-1, :]
    gx[:, :, :-1] = x[:, :, 1:] - x[:, :, :-1]
    if x.shape[0] > 2:
        gz[:-1] = x[1:] - x[:-1]
    return torch.sqrt(gy * gy + gx * gx + gz * gz + beta).sum()
