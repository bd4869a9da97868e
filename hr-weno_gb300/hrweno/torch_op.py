"""Differentiable WENO solves for PyTorch: u(T) = weno_solve(u0, ...) with autograd support.

The forward pass runs the fused FP64 stage kernels; the backward pass is the hand-written
discrete adjoint (hrw_adjoint_vjp), so d(loss)/du0 is the exact gradient of the discrete map
for any loss of u(T).  Problems: FV1D on uniform or non-uniform lines (xedges), global
Lax-Friedrichs at fixed alpha, rktvd order 3; a leading batch of equal-size lines is allowed
(u0 of shape [nseg, ncells] or [ncells]).
"""
from __future__ import annotations

import numpy as np
import torch

from .adjoint import adjoint
from .problems import Problem


class _WenoSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, adj, dt, nsteps):
        u0c = u0.detach().contiguous()
        uT = torch.empty_like(u0c)
        adj.forward(u0c.reshape(-1), None, dt, nsteps, uT=uT.reshape(-1))
        ctx.save_for_backward(u0c)
        ctx.adj, ctx.dt, ctx.nsteps = adj, dt, nsteps
        return uT

    @staticmethod
    def backward(ctx, g):
        (u0c,) = ctx.saved_tensors
        grad = torch.empty_like(u0c)
        ctx.adj.vjp(u0c.reshape(-1), g.contiguous().reshape(-1), ctx.dt, ctx.nsteps,
                    grad=grad.reshape(-1))
        return grad, None, None, None


_cache: dict = {}


def weno_solve(u0: torch.Tensor, problem: Problem, dt: float, nsteps: int,
               checkpoint_every: int = 0) -> torch.Tensor:
    """u(T) after nsteps RK3 steps of dt from u0 (CUDA float64, shape [ncells] or
    [nseg, ncells]), differentiable with respect to u0."""
    if u0.dtype != torch.float64 or not u0.is_cuda:
        raise TypeError("weno_solve needs a CUDA float64 tensor")
    nseg = 1 if u0.dim() == 1 else int(u0.shape[0])
    key = (id(problem), nseg, checkpoint_every, u0.device.index)
    # the descriptor's bytes and the edges of a non-uniform line (the descriptor holds only
    # their address): a problem edited since its handle was made gets a new handle
    snap = bytes(problem.to_c()) + b"".join(
        np.ascontiguousarray(e, dtype=np.float64).tobytes() for e in problem.xedges if e is not None)
    if key not in _cache or _cache[key][1] != snap:
        _cache[key] = (problem, snap, adjoint(problem, nseg=nseg, checkpoint_every=checkpoint_every))
    adj = _cache[key][2]
    return _WenoSolve.apply(u0, adj, float(dt), int(nsteps))
