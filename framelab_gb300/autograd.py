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
    """Gradient of L(x) = 1/2 |A x - b|^2 through the binding vs central
    differences (L(x + h e_i) - L(x - h e_i)) / 2h on n_vox random voxels.

    The loss difference is formed without subtracting two losses or two
    projections: with y = A x and D = A (x + h e_i) - A (x - h e_i),
    L(x + h e_i) - L(x - h e_i) = sum_r D_r (y_r - b_r) exactly, and A is
    linear, so D = A (2 h e_i), the projection of the perturbation alone.
    Each term is then accurate to FP32 rounding. Subtracting the FP32
    projections A (x +- h e_i) instead leaves, on every ray through voxel i,
    the differing rounding of the two walks' running sums after that voxel,
    which at h = 1e-3 is a percent of D_r. The sums run in FP64.
    Returns (max relative error, the checked indices).
    """
    xg = x.detach().clone().requires_grad_(True)
    loss = 0.5 * ((project(xg, plan) - b).double() ** 2).sum()
    loss.backward()
    g = xg.grad.reshape(-1)
    res = (plan.forward(x.detach().contiguous()) - b).double().reshape(-1)
    gen = torch.Generator().manual_seed(seed)
    idx = torch.randperm(x.numel(), generator=gen)[:n_vox]
    e = torch.zeros_like(x.detach()).reshape(-1)
    errs = []
    gscale = g.abs().max().item()
    for i in idx.tolist():
        e[i] = 2.0 * h
        d = plan.forward(e.reshape(x.shape)).double().reshape(-1)
        e[i] = 0.0
        fd = torch.dot(d, res).item() / (2.0 * h)
        errs.append(abs(fd - g[i].item()) / max(abs(g[i].item()), 1e-3 * gscale))
    return max(errs), idx
