"""Native CGLS over the C ABI (Optimizers.CGLS / solveCGLS.m mirror).

``NativeCGLS(plan, mode)`` owns the device workspace; ``solve`` runs
(A^T A + lam I) u = b entirely on the GPU. ``mode='plain'`` is the FP32,
host-synchronised form; ``mode='mixed'`` keeps the search direction in scaled
FP16 for the projector, fuses the vector updates, replays one iteration as a
CUDA graph and refreshes the FP32 residual every ``refresh`` iterations.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

MODES = {"plain": 0, "mixed": 1, "graph": 2}
ZERO_START = 1


def _stream():
    return torch.cuda.current_stream().cuda_stream


def dot(a: torch.Tensor, b: torch.Tensor) -> float:
    """FP64 inner product of two float32 device tensors (ObjectData.objdot)."""
    L = _lib.load()
    out = torch.zeros(1, dtype=torch.float64, device=a.device)
    _lib.check(L.fl_dot(a.data_ptr(), b.data_ptr(), a.numel(), out.data_ptr(), _stream()))
    return float(out.item())


def normal_apply(plan, x: torch.Tensor, lam: float = 0.0, out=None) -> torch.Tensor:
    """(A^T A + lam I) x, matched model, FP32."""
    L = _lib.load()
    out = torch.empty_like(x) if out is None else out
    _lib.check(L.fl_normal_apply(plan.handle, x.data_ptr(), out.data_ptr(), float(lam), _stream()))
    return out


class NativeCGLS:
    def __init__(self, plan, mode: str = "mixed"):
        L = _lib.load()
        self.plan, self.mode = plan, mode
        h = C.c_void_p()
        _lib.check(L.fl_cgls_create(plan.handle, MODES[mode], C.byref(h)))
        self._h, self._L = h, L
        self.history = []
        self.iters_done = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.fl_cgls_destroy(h)
            self._h = None

    def solve(self, b: torch.Tensor, u0: torch.Tensor | None = None, lam: float = 0.0,
              iters: int = 20, tol: float = 1e-14, refresh: int = 10,
              zero_start: bool | None = None) -> torch.Tensor:
        if u0 is None:
            u = torch.zeros_like(b)
            zero_start = True if zero_start is None else zero_start
        else:
            u = u0.clone()
        flags = ZERO_START if zero_start else 0
        hist = np.zeros(max(iters, 1), np.float64)
        nd = C.c_int()
        st = self._L.fl_cgls_solve(self._h, b.data_ptr(), u.data_ptr(), float(lam), int(iters),
                                   float(tol), int(refresh), flags, hist.ctypes.data,
                                   C.byref(nd), _stream())
        self.iters_done = nd.value            # also set when the solve stopped on an error
        self.history = hist[:nd.value].tolist()
        _lib.check(st)
        return u

    def solve_host(self, b: np.ndarray, u: np.ndarray, lam: float = 0.0, iters: int = 20,
                   tol: float = 1e-14, refresh: int = 10, zero_start: bool = True) -> np.ndarray:
        """Host-buffer solve (pinned or pageable numpy float32 arrays); u is overwritten.
        Pinned arrays (e.g. ``torch.empty(n, pin_memory=True).numpy()``) with a
        z-mirror plan in the graph or mixed form are read and written in place
        by the solve's fold kernels; other arrays are copied."""
        hist = np.zeros(max(iters, 1), np.float64)
        nd = C.c_int()
        st = self._L.fl_cgls_solve_host(self._h, b.ctypes.data, u.ctypes.data, float(lam),
                                        int(iters), float(tol), int(refresh),
                                        ZERO_START if zero_start else 0, hist.ctypes.data,
                                        C.byref(nd), _stream())
        self.iters_done = nd.value
        self.history = hist[:nd.value].tolist()
        _lib.check(st)
        return u
