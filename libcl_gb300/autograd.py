"""torch.autograd wrapper of the 3D step's adjoint (gbsph_adjoint3d_*).

`rollout(adj, pos0, vel0, stiffness, viscosity)` sets the fluid's state and gas constant /
viscosity, runs the adjoint's forward (its `steps` steps) and returns the final positions and
velocities; their gradients flow back to pos0, vel0, stiffness and viscosity through the
hand-written CUDA adjoint. PyTorch provides the tape and the tensors; every step and every
derivative runs in libgbsph.so.
"""
from __future__ import annotations

import torch

from . import Adjoint3D, params_derive


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos0, vel0, stiffness, viscosity, adj: Adjoint3D):
        fluid = adj.fluid
        prm = fluid.getParameters()
        prm.stiffness = float(stiffness)
        prm.viscosity = float(viscosity)
        params_derive(prm)
        pos = fluid.getPositionBuffer()
        vel = fluid.getVelocityBuffer()
        pos.copy_(pos0)
        vel.copy_(vel0)
        # the force buffer starts as every step leaves it: the gravity vector
        fluid.getForceBuffer().copy_(torch.tensor(list(prm.gravity), dtype=torch.float32).expand_as(pos))
        adj.forward()
        ctx.adj = adj
        ctx.dtypes = (stiffness.dtype, viscosity.dtype)
        return pos.clone(), vel.clone()

    @staticmethod
    def backward(ctx, g_pos, g_vel):
        adj = ctx.adj
        g_pos = torch.zeros_like(adj.fluid.getPositionBuffer()) if g_pos is None else g_pos.contiguous()
        gp0, gv0, gpar = adj.backward(g_pos, None if g_vel is None else g_vel.contiguous())
        gk = gpar[0].to(ctx.dtypes[0])
        gmu = gpar[1].to(ctx.dtypes[1])
        return gp0, gv0, gk, gmu, None


def rollout(adj: Adjoint3D, pos0: torch.Tensor, vel0: torch.Tensor, stiffness: torch.Tensor,
            viscosity: torch.Tensor):
    """Final (positions, velocities), float32 [N, 4] each, after `adj.steps` steps from
    (pos0, vel0) with the given gas constant and viscosity (0-d tensors). Differentiable in
    pos0, vel0 (.w lanes get zero gradient), stiffness and viscosity."""
    return _Rollout.apply(pos0, vel0, stiffness, viscosity, adj)
