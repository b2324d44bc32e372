"""torch.autograd bridge of the checkpointed adjoint.

``evolve(prim0, nsteps, ...)`` runs the FP64 solver for ``nsteps`` steps and
returns the final primitive state as a tensor that carries a gradient: its
backward pass is the hand-written reverse mode of the time step behind the C
ABI (eulr_adjoint_*), not torch autograd of any torch operation.  dt is held
fixed at the forward sequence (the CFL steps the forward pass took, or the
given ``dts``).
"""
from __future__ import annotations

import torch

from . import Adjoint


class _Evolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, prim0, nsteps, gamma, dx, cfl, dts, checkpoint_every):
        if prim0.dtype != torch.float64 or not prim0.is_cuda:
            raise TypeError("evolve needs a float64 CUDA tensor of shape (5, n2, n1, n0)")
        prim0 = prim0.contiguous()
        n2, n1, n0 = prim0.shape[1:]
        stream = torch.cuda.current_stream(prim0.device)
        adj = Adjoint(n0, n1, n2, nsteps, gamma=gamma, dx=dx, cfl=cfl, checkpoint_every=checkpoint_every,
                      stream=stream)
        out = torch.empty_like(prim0)
        adj.forward(prim0, dts=dts, out=out)
        ctx.adj = adj
        return out

    @staticmethod
    def backward(ctx, grad_out):
        grad_out = grad_out.contiguous()
        grad0 = torch.empty_like(grad_out)
        ctx.adj.backward(grad_out, grad0)
        return grad0, None, None, None, None, None, None


def evolve(prim0: torch.Tensor, nsteps: int, gamma: float = 1.4, dx=None, cfl: float = 0.4, dts=None,
           checkpoint_every: int = 20) -> torch.Tensor:
    """Final primitive state after ``nsteps`` steps from ``prim0``; differentiable.

    ``dx`` defaults to the unit cube (1/(n-2) per axis).  ``dts`` (a sequence of
    ``nsteps`` step lengths) fixes dt; otherwise the CFL steps of the forward
    pass are recorded and held fixed for the gradient."""
    if dx is None:
        n2, n1, n0 = prim0.shape[1:]
        dx = (1.0 / (n0 - 2), 1.0 / (n1 - 2), 1.0 / (n2 - 2))
    return _Evolve.apply(prim0, int(nsteps), float(gamma), tuple(float(v) for v in dx), float(cfl),
                         None if dts is None else [float(v) for v in dts], int(checkpoint_every))
