"""torch.autograd.Function over the hand-written adjoint (include/fqsb.h, fqsb_adjoint_*).

    loss = TrajectoryLoss.apply(system, u0, v0, schedule, params, K, last)

runs the system from (u0, v0, a = 0) for len(schedule) steps with u_frame = schedule[t] before step t
and returns L = mean over the last `last` steps of mean(f_frame) + 0.5 mean(u_T^2); params is the
tensor [mu, k_interactions, eta].  loss.backward() gives the gradients with respect to u0, v0,
schedule and params from the adjoint kernel (checkpoints every K steps, recomputation of each
segment).  Exact for Smooth and SemiSmooth potentials; Cuspy holds the wells of the forward.
PyTorch is only the autograd plumbing: all arithmetic runs in the library's FP64 kernels.

CUDA tensors on the system's device stay on the device: u0 and v0 are copied into the system with
fqsb_set_field_device and the gradients dL/du0, dL/dv0 are written into device tensors by
fqsb_adjoint_backward_device; only the schedule (len(schedule) doubles), the three parameters and
the scalar loss cross to the host.  Other tensors go through host arrays.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _capi as C


def _on_system_device(system, t: torch.Tensor) -> bool:
    return t.is_cuda and t.device.index == system.device


def _set_state(system, field: int, t: torch.Tensor):
    if _on_system_device(system, t):
        x = t.detach().to(torch.float64).contiguous()
        if x.numel() != system.size:
            raise ValueError(f"expected {system.size} values, got {x.numel()}")
        # the library's stream reads x: finish the work that produced it on torch's stream first
        torch.cuda.current_stream(x.device).synchronize()
        system.set_field_device(field, x.data_ptr())
    else:
        arr = t.detach().cpu().numpy().astype(np.float64).reshape(system.shape)
        if field == C.FIELD_U:
            system.u = arr
        else:
            system.v = arr


class TrajectoryLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, system, u0, v0, schedule, params, K=100, last=500):
        mu, k, eta = [float(x) for x in params.detach().cpu().tolist()]
        system.set_parameters(mu, k, eta)
        _set_state(system, C.FIELD_U, u0)
        _set_state(system, C.FIELD_V, v0)
        system.a = np.zeros(system.shape)
        loss = system.adjoint_forward(schedule.detach().cpu().numpy().astype(np.float64), K=K, last=last)
        ctx.system = system
        ctx.meta = [(t.device, t.shape) for t in (u0, v0, schedule, params)]
        return torch.tensor(loss, dtype=torch.float64, device=u0.device)

    @staticmethod
    def backward(ctx, grad):
        system = ctx.system
        (du, su), (dv, sv), (ds, _), (dp, _) = ctx.meta
        g = float(grad.detach().cpu().item())
        if du.type == "cuda" and du.index == system.device and dv.type == "cuda" and dv.index == system.device:
            gu = torch.empty(system.size, dtype=torch.float64, device=du)
            gv = torch.empty(system.size, dtype=torch.float64, device=dv)
            gs, gp = system.adjoint_backward_device(gu.data_ptr(), gv.data_ptr())
            gu = (gu * g).reshape(su)
            gv = (gv * g).reshape(sv)
        else:
            hu, hv, gs, gp = system.adjoint_backward()
            gu = torch.from_numpy(g * hu).to(du).reshape(su)
            gv = torch.from_numpy(g * hv).to(dv).reshape(sv)
        return (None, gu, gv, torch.from_numpy(g * gs).to(ds), torch.from_numpy(g * gp).to(dp), None, None)


def trajectory_loss(system, u0, v0, schedule, params, K=100, last=500):
    return TrajectoryLoss.apply(system, u0, v0, schedule, params, K, last)
