"""Differentiable rollouts: gradients of a loss on the final particle state
with respect to per-particle Young's modulus and initial velocity, through the
hand-written adjoint kernels (mpm_fwd_checkpointed / mpm_bwd).

``Rollout`` is a torch.autograd.Function -- the Python counterpart of the
ChainRulesCore.rrule a Julia binding would define -- mapping (E, v0) to the
final positions of every particle of a problem:

    x = Rollout.apply(E, v0, problem, nsteps, checkpoint_every)
    loss = ((x[tip] - target) ** 2).sum()
    loss.backward()        # E.grad, v0.grad from the adjoint sweep

``problem`` is the (grid, solids, alg, data) tuple of a solver call; E and v0
replace ``solids[*].youngs`` and ``solids[*].velocity`` (all bodies in order).
"""
from __future__ import annotations

import copy

import numpy as np

from .dirichlet import fix_Dirichlet_grid
from .engine import Descriptors, MPMContext


def make_context(problem, E=None, v0=None):
    """A context for problem with per-particle E and initial velocity v0 substituted."""
    grid, solids, alg, data = problem
    solids = copy.deepcopy(solids)
    off = 0
    for s in solids:
        n = s.parCount
        if E is not None:
            s.youngs = np.asarray(E[off:off + n], dtype=np.float64).copy()
        if v0 is not None:
            s.velocity = np.asarray(v0[off:off + n], dtype=np.float64).reshape(n, s.dim).copy()
        off += n
    fix_Dirichlet_grid(grid, data, ghostcell="ghostcell" in data)
    d = Descriptors(grid, solids, tolerance=alg.tolerance, body_force=data.get("bodyforce"), dt=data["dt"])
    return MPMContext(d)


def final_positions(ctx) -> np.ndarray:
    return np.concatenate([s.pos for s in ctx.download_all()])


def rollout_grad(problem, E, v0, nsteps, every, loss_grad):
    """Run forward with checkpoints, return (x_final, gradient dict) for
    dL/dx_final = loss_grad(x_final)."""
    ctx = make_context(problem, E, v0)
    ctx.fwd_checkpointed(nsteps, every)
    x = final_positions(ctx)
    g = ctx.bwd(loss_grad(x))
    ctx.close()
    return x, g


try:
    import torch

    class Rollout(torch.autograd.Function):
        """(E, v0) -> final positions, with the adjoint sweep as backward."""

        @staticmethod
        def forward(fctx, E, v0, problem, nsteps, every):
            c = make_context(problem, E.detach().cpu().numpy(), v0.detach().cpu().numpy())
            c.fwd_checkpointed(int(nsteps), int(every))
            fctx.mpm = c
            return torch.from_numpy(final_positions(c)).to(E.dtype)

        @staticmethod
        def backward(fctx, grad_x):
            g = fctx.mpm.bwd(grad_x.detach().cpu().numpy().astype(np.float64))
            fctx.mpm.close()
            return (torch.from_numpy(g["E"]).to(grad_x.dtype), torch.from_numpy(g["v0"]).to(grad_x.dtype),
                    None, None, None)
except ImportError:  # torch is optional for the C/Python API
    Rollout = None
