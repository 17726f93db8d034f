"""torch.autograd binding of the MLS transfer (test binding of the adjoint).

``mls_transfer(source_values, source_points, target_points, rbf, basis, k=...)``
builds the operator on the given points, applies it, and on backward calls
the library's adjoint (``dtk_mls_apply_adjoint``): the gradient with respect
to the source values is C^T g (deterministic transpose gather) and the
gradient with respect to the source coordinates goes through the RBF weights,
the support radius and the pseudo-inverse, recomputed per target.  The
neighbour sets are piecewise constant in the coordinates and carry no
gradient.  Gradients with respect to the target points are not provided.
"""
from __future__ import annotations

import torch

from .operators import MovingLeastSquaresOperator


class MLSTransferFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, source_values, source_points, target_points, rbf, basis, k, radius, precision):
        op = MovingLeastSquaresOperator(None, source_points.detach(), target_points.detach(), rbf, basis,
                                        k=k, radius=radius, precision=precision, keep_points=True)
        sv = source_values.detach().contiguous()
        out = torch.empty(target_points.shape[0], dtype=torch.float64, device=source_values.device)
        op.apply(sv, out)
        ctx.op = op
        ctx.save_for_backward(sv)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        if ctx.needs_input_grad[2]:
            raise NotImplementedError("the MLS adjoint has no gradient with respect to the target points")
        (sv,) = ctx.saved_tensors
        want_coords = ctx.needs_input_grad[1]
        gv, gc = ctx.op.apply_adjoint(grad_out.contiguous(), sv if want_coords else None,
                                      coords=want_coords)
        return (gv if ctx.needs_input_grad[0] else None, gc, None, None, None, None, None, None)


def mls_transfer(source_values, source_points, target_points, rbf=None, basis=None, *, k=None,
                 radius=None, precision="fp64"):
    """Differentiable MLS transfer of ``source_values`` onto ``target_points``."""
    return MLSTransferFunction.apply(source_values, source_points, target_points, rbf, basis, k, radius,
                                     precision)
