"""PyTorch autograd over the engine's hand-written adjoint.

``structure_factor_rollout(psi0, eps, k, M, params, nsteps)`` runs `nsteps`
time steps of a 2D Landau box from `psi0` with the given (epsilon, k, M) and
returns the radially averaged S(q) of the final state (the definition of the
reference's utils/sq_from_traj.py).  Its backward pass is the engine's
adjoint (chgb_adjoint_backward), so any loss built on S(q) in PyTorch gets
dL/dpsi0 and dL/d(epsilon, k, M) without storing the trajectory.
"""
from __future__ import annotations

import numpy as np
import torch

from . import abi
from .sim import Adjoint


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, psi0, eps, k, M, params, nsteps, checkpoint_every):
        p = params.copy()
        p.model.epsilon = float(eps)
        p.k[0] = float(k)
        p.M = float(M)
        adj = Adjoint(p, nsteps, checkpoint_every)
        sq, _ = adj.forward(psi0.detach().to("cpu", torch.float64).numpy())
        ctx.adj = adj
        ctx.shape = psi0.shape
        ctx.device = psi0.device
        return torch.from_numpy(sq).to(psi0.device)

    @staticmethod
    def backward(ctx, grad_sq):
        g0, g3 = ctx.adj.backward(dl_dsq=grad_sq.detach().to("cpu", torch.float64).numpy())
        ctx.adj.close()
        dev = ctx.device
        as_t = lambda v: torch.tensor(v, dtype=torch.float64, device=dev)  # noqa: E731
        return (torch.from_numpy(g0).reshape(ctx.shape).to(dev), as_t(g3[0]), as_t(g3[1]), as_t(g3[2]),
                None, None, None)


def structure_factor_rollout(psi0: torch.Tensor, eps: torch.Tensor, k: torch.Tensor, M: torch.Tensor,
                             params: abi.Params, nsteps: int, checkpoint_every: int = 0) -> torch.Tensor:
    """S(q) after `nsteps` steps; differentiable in psi0, eps, k and M."""
    return _Rollout.apply(psi0, eps, k, M, params, int(nsteps), int(checkpoint_every))


def sq_loss(sq: torch.Tensor, target: torch.Tensor) -> torch.Tensor:
    """sum_q (S(q) - S*(q))^2."""
    return torch.sum((sq - target) ** 2)


__all__ = ["structure_factor_rollout", "sq_loss", "np"]
