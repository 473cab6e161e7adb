"""torch.autograd.Function over the trajectory adjoint of a DiffSystem: the
forward runs the trajectory on the GPU (mrmd_diff_forward), the backward the
hand-written adjoint sweep (mrmd_diff_backward).  A thin shim: the compute is
in libmrmd_gb300.so."""
from __future__ import annotations

import torch


class TrajectoryLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, table, epsilon, sigma, system):
        loss = system.forward(table.detach().cpu().double().numpy(), float(epsilon), float(sigma))
        ctx.system = system
        ctx.meta = (table.dtype, table.device, epsilon.dtype, epsilon.device)
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        gt, ge, gs = ctx.system.backward()
        g = float(grad_out)
        tdt, tdev, edt, edev = ctx.meta
        return (torch.from_numpy(gt * g).to(dtype=tdt, device=tdev),
                torch.tensor(ge * g, dtype=edt, device=edev),
                torch.tensor(gs * g, dtype=edt, device=edev), None)


def trajectory_loss(system, table, epsilon, sigma):
    """Loss of the trajectory with TF table `table` and LJ epsilon, sigma
    (tensors); differentiable with respect to all three."""
    return TrajectoryLoss.apply(table, epsilon, sigma, system)
