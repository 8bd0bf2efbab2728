"""torch.autograd binding of the adjoint (ch_adjoint).

    import torch, importlib
    chy = importlib.import_module("collisional-hybrid_gb300")
    from importlib import import_module
    ag = import_module("collisional-hybrid_gb300.autograd")
    adj = chy.Adjoint(params, nions, loader, nsteps=50, checkpoint_every=10, window=10)
    theta = torch.tensor(adj.theta0(), dtype=torch.float64, requires_grad=True)
    J = ag.objective(theta, adj)       # forward run, collision events recorded
    J.backward()                       # reverse sweep on the GPU
    theta.grad                         # dJ/d(E0, vn0, amp)

The forward records (freezes) the collision events at the given theta; the
gradient is exact for that frozen-event model.  theta lives on the host (7
FP64 scalars); the state of the run stays on the GPU inside `adj`.
"""
from __future__ import annotations

import numpy as np
import torch


class HybridObjective(torch.autograd.Function):
    """J(theta) of a ch_adjoint run; backward = its discrete adjoint."""

    @staticmethod
    def forward(ctx, theta: torch.Tensor, adj) -> torch.Tensor:
        th = theta.detach().to("cpu", torch.float64).numpy()
        J = adj.forward(th, record=True)
        ctx.adj = adj
        ctx.device = theta.device
        return torch.tensor(J, dtype=torch.float64, device=theta.device)

    @staticmethod
    def backward(ctx, gJ: torch.Tensor):
        g, _ = ctx.adj.gradient()
        grad = torch.from_numpy(np.ascontiguousarray(g)).to(ctx.device)
        return gJ * grad, None


def objective(theta: torch.Tensor, adj) -> torch.Tensor:
    return HybridObjective.apply(theta, adj)
