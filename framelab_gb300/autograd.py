"""torch.autograd binding of the matched projector pair (test harness use).

``project(x, plan)`` is y = A x with backward x_grad = A^T y_grad, where A^T is
the library's exact-transpose backprojector, so gradients of any loss of the
projections (e.g. 1/2 |A x - b|^2) come out of the same matrix.
"""
from __future__ import annotations

import torch


class Project(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x: torch.Tensor, plan) -> torch.Tensor:
        ctx.plan = plan
        ctx.x_shape = x.shape
        return plan.forward(x.detach().contiguous())

    @staticmethod
    def backward(ctx, gy: torch.Tensor):
        return ctx.plan.adjoint(gy.detach().contiguous()).reshape(ctx.x_shape), None


def project(x: torch.Tensor, plan) -> torch.Tensor:
    return Project.apply(x, plan)


def fd_gradcheck(plan, x: torch.Tensor, b: torch.Tensor, n_vox: int = 64, h: float = 1e-3,
                 seed: int = 0):
    """Gradient of 1/2 |A x - b|^2 through the binding vs central differences
    (h) on n_vox random voxels. The loss is accumulated in FP64 from the FP32
    projections. Returns (max relative error, the checked indices)."""
    xg = x.detach().clone().requires_grad_(True)
    loss = 0.5 * ((project(xg, plan) - b).double() ** 2).sum()
    loss.backward()
    g = xg.grad.reshape(-1)
    gen = torch.Generator().manual_seed(seed)
    idx = torch.randperm(x.numel(), generator=gen)[:n_vox]
    flat = x.detach().reshape(-1).clone()

    def f(v):
        return 0.5 * ((plan.forward(v.reshape(x.shape)) - b).double() ** 2).sum().item()

    errs = []
    gscale = g.abs().max().item()
    for i in idx.tolist():
        old = flat[i].item()
        flat[i] = old + h
        fp = f(flat)
        flat[i] = old - h
        fm = f(flat)
        flat[i] = old
        fd = (fp - fm) / (2 * h)
        errs.append(abs(fd - g[i].item()) / max(abs(g[i].item()), 1e-3 * gscale))
    return max(errs), idx
