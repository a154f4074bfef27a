"""torch.autograd bindings of the flux residual: the forward / VJP pair of the
C ABI (qlskum_residual_forward, qlskum_residual_vjp) as an
autograd.Function, so a PyTorch graph can differentiate through R(prim).

The library takes host buffers; tensors are moved to the CPU in FP64 for the
call and the result is returned on the input's device and dtype.
"""
from __future__ import annotations

import numpy as np
import torch


class FluxResidual(torch.autograd.Function):
    """R = FluxResidual.apply(prim, solver): prim [n, 4] (rho, u1, u2, p)."""

    @staticmethod
    def forward(ctx, prim: torch.Tensor, solver) -> torch.Tensor:
        p = prim.detach().to("cpu", torch.float64).contiguous().numpy()
        ctx.solver = solver
        ctx.save_for_backward(prim.detach())
        out = solver.residual(p)
        return torch.from_numpy(out).to(prim.device, prim.dtype)

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        (prim,) = ctx.saved_tensors
        p = prim.to("cpu", torch.float64).contiguous().numpy()
        g = grad_out.detach().to("cpu", torch.float64).contiguous().numpy()
        bar = ctx.solver.residual_vjp(p, g)
        return torch.from_numpy(np.ascontiguousarray(bar)).to(prim.device, prim.dtype), None


def flux_residual(prim: torch.Tensor, solver) -> torch.Tensor:
    return FluxResidual.apply(prim, solver)
