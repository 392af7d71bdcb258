"""torch.autograd wrapper of a GPU rollout, for checking gradients with torch
tools (gradcheck, optimisers).  The forward runs ``nsteps`` steps of a
program on a :class:`formura_gb300.host.Grid`; the backward runs the
checkpointed reverse sweep of the runtime (``fgb_gradient_*``).
"""
from __future__ import annotations

import numpy as np
import torch

from .host import Grid


class Rollout(torch.autograd.Function):
    """u_T = step^nsteps(u_0) on the GPU; gradient by the generated adjoint."""

    @staticmethod
    def forward(ctx, u0: torch.Tensor, grid: Grid, nsteps: int, snapshots: int):
        x = u0.detach().to("cpu", torch.float64).contiguous().numpy()
        grid.upload(x)
        grid.forward(nsteps)
        uT = grid.download()
        ctx.grid, ctx.u0, ctx.nsteps, ctx.snapshots = grid, x, nsteps, snapshots
        ctx.dtype, ctx.device = u0.dtype, u0.device
        return torch.from_numpy(uT).to(u0.device, u0.dtype)

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        # each backward records its own checkpointed forward pass, so the
        # graph may be differentiated more than once (gradcheck does)
        g = ctx.grid
        g.upload(ctx.u0)
        g.gradient_forward(ctx.nsteps, ctx.snapshots)
        grad = g.gradient_backward(grad_out.detach().to("cpu", torch.float64).contiguous().numpy())
        return torch.from_numpy(grad).to(ctx.device, ctx.dtype), None, None, None


def rollout(u0: torch.Tensor, grid: Grid, nsteps: int, snapshots: int = 8) -> torch.Tensor:
    return Rollout.apply(u0, grid, nsteps, snapshots)
