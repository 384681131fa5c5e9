"""Framelets and split Bregman over the C ABI (Transforms.FrameletSystem,
Optimizers.SplitBregman mirrors).

Coefficient sets are flat float32 device tensors of ``ncoef`` elements:
level-major, bands in pass order (3-D: index 9i + 3j + k for D_i along y,
D_j along x, D_k along z; 2-D: 3i + j for D_i along x, D_j along y), each band
one volume; the low band of every level but the last is not stored (the
reference's synthesis never reads it).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

_V = C.c_void_p
KINDS = {"haar": 0, "linear": 1, "cubic": 3}


def _stream():
    return torch.cuda.current_stream().cuda_stream


class FrameletSystem:
    """FrameletSystem(dim, type, level) on an nx*ny(*nz) grid (FrameletSystem.m:12-64)."""

    def __init__(self, shape, kind: str = "linear", levels: int = 1):
        L = _lib.load()
        shape = tuple(int(s) for s in shape)
        if len(shape) == 2:
            ny, nx = shape; nz = 1
        else:
            nz, ny, nx = shape
        self.shape, self.kind, self.levels = shape, kind, levels
        h = C.c_void_p()
        _lib.check(L.fl_framelet_create(nx, ny, nz, levels, KINDS[kind], C.byref(h)))
        self._h, self._L = h, L
        self._fused = True
        self.ncoef = int(L.fl_framelet_ncoef(h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.fl_framelet_destroy(h)
            self._h = None

    @property
    def fused(self) -> bool:
        """3-D levels through the fused tile kernels (default) or the separable passes."""
        return self._fused

    @fused.setter
    def fused(self, on: bool):
        _lib.check(self._L.fl_framelet_option(self._h, _lib.FRAMELET_OPT_FUSED, int(bool(on))))
        self._fused = bool(on)

    def forward(self, u: torch.Tensor) -> torch.Tensor:
        out = torch.empty(self.ncoef, device=u.device, dtype=torch.float32)
        _lib.check(self._L.fl_framelet_analysis(self._h, u.data_ptr(), out.data_ptr(), _stream()))
        return out

    def adjoint(self, coef: torch.Tensor) -> torch.Tensor:
        out = torch.empty(self.shape, device=coef.device, dtype=torch.float32)
        _lib.check(self._L.fl_framelet_synthesis(self._h, coef.data_ptr(), out.data_ptr(),
                                                 _stream()))
        return out

    def bregman(self, u, v, t, Atf, mu, tau, b):
        _lib.check(self._L.fl_framelet_bregman(self._h, u.data_ptr(), v.data_ptr(), t.data_ptr(),
                                               Atf.data_ptr() if Atf is not None else None,
                                               float(mu), float(tau), b.data_ptr(), _stream()))
        return b


class SplitBregmanSolver:
    """Device split Bregman on one plan with a persistent workspace
    (fl_sb_create / fl_sb_run): the framelet, CGLS workspace and coefficient
    sets are allocated once and reused by every solve."""

    def __init__(self, plan, levels: int = 2, kind: str = "linear", mode: str = "mixed"):
        from .solvers import MODES
        L = _lib.load()
        h = C.c_void_p()
        _lib.check(L.fl_sb_create(plan.handle, int(levels), KINDS[kind], MODES[mode], C.byref(h)))
        self.plan, self._h, self._L = plan, h, L
        self.history = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.fl_sb_destroy(h)
            self._h = None

    def solve(self, f: torch.Tensor, u0: torch.Tensor, lam: float, mu: float, outer: int = 30,
              cg_iters: int = 5, cg_tol: float = 1e-10) -> torch.Tensor:
        u = u0.clone()
        hist = np.zeros(max(outer, 1), np.float64)
        _lib.check(self._L.fl_sb_run(self._h, f.data_ptr(), u.data_ptr(), float(lam), float(mu),
                                     int(outer), int(cg_iters), float(cg_tol), hist.ctypes.data,
                                     _stream()))
        self.history = hist[:outer]
        return u


def split_bregman(plan, f: torch.Tensor, u0: torch.Tensor, lam: float, mu: float,
                  outer: int = 30, cg_iters: int = 5, cg_tol: float = 1e-10, levels: int = 2,
                  kind: str = "linear", mode: str = "mixed"):
    """solveSplitBregman.m on the device; returns (u, history)."""
    from .solvers import MODES
    L = _lib.load()
    u = u0.clone()
    hist = np.zeros(max(outer, 1), np.float64)
    _lib.check(L.fl_sb_solve(plan.handle, f.data_ptr(), u.data_ptr(), float(lam), float(mu),
                             int(outer), int(cg_iters), float(cg_tol), int(levels), KINDS[kind],
                             MODES[mode], hist.ctypes.data, _stream()))
    return u, hist[:outer]
