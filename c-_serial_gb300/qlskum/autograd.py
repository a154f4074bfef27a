"""torch.autograd bindings of the flux residual: the forward / VJP pair of the
C ABI as an autograd.Function, so a PyTorch graph can differentiate through
R(prim).

CUDA tensors go through qlskum_residual_forward_device /
qlskum_residual_vjp_device: FP64 device buffers in the cloud's point order,
ordered on the current torch stream, with no host copy.  CPU tensors go
through the host-buffer pair (qlskum_residual_forward, qlskum_residual_vjp).
Results come back on the input's device and dtype.
"""
from __future__ import annotations

import numpy as np
import torch


def _dev64(t: torch.Tensor) -> torch.Tensor:
    return t.detach().to(torch.float64).contiguous()


class FluxResidual(torch.autograd.Function):
    """R = FluxResidual.apply(prim, solver): prim [n, 4] (rho, u1, u2, p)."""

    @staticmethod
    def forward(ctx, prim: torch.Tensor, solver) -> torch.Tensor:
        ctx.solver = solver
        ctx.save_for_backward(prim.detach())
        if prim.is_cuda:
            p = _dev64(prim)
            out = torch.empty_like(p)
            solver.residual_device(p.data_ptr(), out.data_ptr(), torch.cuda.current_stream(p.device).cuda_stream)
            return out.to(prim.dtype)
        p = prim.detach().to("cpu", torch.float64).contiguous().numpy()
        out = solver.residual(p)
        return torch.from_numpy(out).to(prim.device, prim.dtype)

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        (prim,) = ctx.saved_tensors
        solver = ctx.solver
        if prim.is_cuda:
            p = _dev64(prim)
            g = _dev64(grad_out.to(prim.device))
            bar = torch.empty_like(p)
            solver.residual_vjp_device(p.data_ptr(), g.data_ptr(), bar.data_ptr(),
                                       torch.cuda.current_stream(p.device).cuda_stream)
            return bar.to(prim.dtype), None
        p = prim.to("cpu", torch.float64).contiguous().numpy()
        g = grad_out.detach().to("cpu", torch.float64).contiguous().numpy()
        bar = solver.residual_vjp(p, g)
        return torch.from_numpy(np.ascontiguousarray(bar)).to(prim.device, prim.dtype), None


def flux_residual(prim: torch.Tensor, solver) -> torch.Tensor:
    return FluxResidual.apply(prim, solver)
