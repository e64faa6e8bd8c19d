"""torch.autograd.Function over the hand-written adjoint (include/fqsb.h, fqsb_adjoint_*).

    loss = TrajectoryLoss.apply(system, u0, v0, schedule, params, K, last)

runs the system from (u0, v0, a = 0) for len(schedule) steps with u_frame = schedule[t] before step t
and returns L = mean over the last `last` steps of mean(f_frame) + 0.5 mean(u_T^2); params is the
tensor [mu, k_interactions, eta].  loss.backward() gives the gradients with respect to u0, v0,
schedule and params from the adjoint kernel (checkpoints every K steps, recomputation of each
segment).  Exact for Smooth and SemiSmooth potentials; Cuspy holds the wells of the forward.
PyTorch is only the autograd plumbing: all arithmetic runs in the library's FP64 kernels.
"""

from __future__ import annotations

import numpy as np
import torch


class TrajectoryLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, system, u0, v0, schedule, params, K=100, last=500):
        mu, k, eta = [float(x) for x in params.detach().cpu().tolist()]
        system.set_parameters(mu, k, eta)
        system.u = u0.detach().cpu().numpy().astype(np.float64)
        system.v = v0.detach().cpu().numpy().astype(np.float64)
        system.a = np.zeros(system.shape)
        loss = system.adjoint_forward(schedule.detach().cpu().numpy().astype(np.float64), K=K, last=last)
        ctx.system = system
        ctx.devices = (u0.device, v0.device, schedule.device, params.device)
        return torch.tensor(loss, dtype=torch.float64, device=u0.device)

    @staticmethod
    def backward(ctx, grad):
        gu, gv, gs, gp = ctx.system.adjoint_backward()
        g = grad.detach().cpu().item()
        du, dv, ds, dp = ctx.devices
        return (None,
                torch.from_numpy(g * gu).to(du),
                torch.from_numpy(g * gv).to(dv),
                torch.from_numpy(g * gs).to(ds),
                torch.from_numpy(g * gp).to(dp),
                None, None)


def trajectory_loss(system, u0, v0, schedule, params, K=100, last=500):
    return TrajectoryLoss.apply(system, u0, v0, schedule, params, K, last)
