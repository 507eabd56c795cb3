"""torch.autograd bridge to md_adjoint_run, for checking only.

``TrajectoryLoss.apply(lj1, lj2, lns, build)`` evaluates the trajectory loss
of a batch built by ``build(lj1, lj2, charge_scale)`` (a callable returning a
fresh MDSystem batch) and returns the per-replica losses; its backward pass
hands torch the adjoint gradients the library computed in the same run.
The library does all the work on the GPU; this wrapper only routes tensors.
"""
from __future__ import annotations

import numpy as np


def _torch():
    import torch
    return torch


def make_function():
    torch = _torch()

    class TrajectoryLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, lj1, lj2, lns, build, kwargs):
            sim = build(lj1.detach().cpu().numpy(), lj2.detach().cpu().numpy(),
                        float(np.exp(lns.detach().cpu().item())))
            try:
                out = sim.adjoint(gradient=True, **kwargs)
            finally:
                sim.close()
            nt = lj1.shape[-1]
            ctx.save_for_backward(torch.as_tensor(out["dlj1"][:, :nt, :nt]),
                                  torch.as_tensor(out["dlj2"][:, :nt, :nt]),
                                  torch.as_tensor(out["dlns"]))
            return torch.as_tensor(out["loss"])

        @staticmethod
        def backward(ctx, grad_loss):
            d1, d2, ds = ctx.saved_tensors
            g = grad_loss.to(d1.dtype)
            # one parameter set shared by all replicas: sum over replicas
            return ((g[:, None, None] * d1).sum(0), (g[:, None, None] * d2).sum(0),
                    (g * ds).sum().reshape(()), None, None)

    return TrajectoryLoss
