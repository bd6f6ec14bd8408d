"""A thin ``torch.autograd.Function`` over the adjoint of the implicit step, for
gradient checks: the trajectory's final positions as a differentiable function of the
per-spring Ks and Kd, the initial velocities and a constant per-vertex external force.

The computation runs in the native library (oc_tape_forward / oc_tape_backward); torch
only carries the CPU tensors in and out.
"""
from __future__ import annotations

import numpy as np
import torch

from .cloth import ClothSolver


class ClothTrajectory(torch.autograd.Function):
    """X_T = f(ks, kd, v0, ext) for a fixed solver handle, X0, dt and step count."""

    @staticmethod
    def forward(ctx, ks, kd, v0, ext, solver: ClothSolver, X0, dt: float, n_steps: int, checkpoint_every: int = 0):
        solver.set_spring_params(ks.detach().cpu().numpy(), kd.detach().cpu().numpy())
        solver.set_ext_force(ext.detach().cpu().numpy())
        X0 = np.asarray(X0, np.float32)
        solver.set_state(X0, v0.detach().cpu().numpy(), np.zeros_like(X0))
        solver.tape_forward(dt, n_steps, checkpoint_every)
        X, _, _ = solver.get_state()
        ctx.solver = solver
        return torch.from_numpy(X)

    @staticmethod
    def backward(ctx, gX):
        g = ctx.solver.tape_backward(gX.detach().cpu().numpy())
        return (torch.from_numpy(g["dKs"]), torch.from_numpy(g["dKd"]), torch.from_numpy(g["dV0"]),
                torch.from_numpy(g["dext"]), None, None, None, None, None)


def trajectory(solver: ClothSolver, X0, ks, kd, v0, ext, dt: float, n_steps: int, checkpoint_every: int = 0):
    return ClothTrajectory.apply(ks, kd, v0, ext, solver, X0, dt, n_steps, checkpoint_every)
