"""torch.autograd wrapper of the operator apply, for checking the
hand-written adjoint only (not a compute path of its own).

forward:  y = A(kappa) x            (sf_vmult)
backward: dL/dx     = A^T dL/dy     (sf_vmult_transpose; A is symmetric)
          dL/dkappa = grad(x) . G grad(dL/dy) per Gauss point
                                    (sf_kappa_gradient, gradients recomputed)
"""
from __future__ import annotations

import torch

from .sfgpu import Operator


class LaplaceApply(torch.autograd.Function):
    @staticmethod
    def forward(ctx, op: Operator, x: torch.Tensor, kappa: torch.Tensor):
        op.set_coefficient(kappa.detach().double().contiguous())
        y = torch.empty_like(x)
        op.vmult(x.detach().contiguous(), y)
        ctx.op = op
        ctx.save_for_backward(x, kappa)
        return y

    @staticmethod
    def backward(ctx, gy):
        x, kappa = ctx.saved_tensors
        op = ctx.op
        op.set_coefficient(kappa.detach().double().contiguous())
        gy = gy.contiguous()
        gx = gk = None
        if ctx.needs_input_grad[1]:
            gx = torch.empty_like(gy)
            op.vmult_transpose(gy, gx)
        if ctx.needs_input_grad[2]:
            gk = torch.empty(kappa.shape, dtype=gy.dtype, device=gy.device)
            op.kappa_gradient(x.detach().contiguous(), gy, gk)
        return None, gx, gk


def laplace_apply(op: Operator, x: torch.Tensor, kappa: torch.Tensor) -> torch.Tensor:
    return LaplaceApply.apply(op, x, kappa)
