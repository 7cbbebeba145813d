"""Test-only harness: the GPU tracer window behind a torch.autograd.Function, its
forward the window's forward sweep and the SST cost, its backward the checkpointed
adjoint sweep (the gradient with the FCT limiter frozen at the forward's values)."""
import torch

from nemo_gpu.adjoint import sst_cost


class WindowCost(torch.autograd.Function):
    """J(t0) for a window started from tsb = tsn = t0 (an Euler start)."""

    @staticmethod
    def forward(ctx, t0, window, target, tmask_surf, shape):
        _, tsn = window.forward(t0, t0)
        J, g = sst_cost(tsn, target, tmask_surf, shape)
        ctx.window = window
        ctx.g = g
        return J

    @staticmethod
    def backward(ctx, gJ):
        w = ctx.window
        ab0, an0 = w.adjoint(torch.zeros_like(ctx.g), ctx.g * gJ)
        return ab0 + an0, None, None, None, None
