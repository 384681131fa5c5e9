"""Batched uneven fan-beam slices over the C ABI (``fl_batch_*``).

``FanBatch(paras)`` takes one fan ``para`` per slice (any mix of image sizes,
detector widths and view counts), builds a :class:`~framelab_gb300.projector.Plan`
per slice and one native batch over them. Images and sinograms of all slices
live concatenated in one device tensor each (slice ``i`` at
``vox_offsets[i]:vox_offsets[i+1]`` / ``ray_offsets[i]:ray_offsets[i+1]``), and
every operator is one kernel launch for the whole batch, or two when some
slices use the half or quarter turn of their plan (they run the plan's turn
kernels). The per-slice results equal the slice plan's own matched
forward/adjoint bit for bit, with the plan's turn options as they were when
the batch was created.

This is the reference's per-slice loop over ``FanBeamScanner.apply`` /
``applyAdjoint`` and ``solveCGLS`` (``solveCGLS.m:6-31``) as one batched solve.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .projector import Plan

ZERO_START = 1


def _stream():
    return torch.cuda.current_stream().cuda_stream


class FanBatch:
    """Many single-frame fan-beam scans projected and solved together."""

    def __init__(self, paras, turns: bool = True, fan_parts: int | None = None,
                 reflect: bool = True):
        """``turns=False`` keeps every slice on the general kernels (each
        plan's half / quarter turn and reflection switched off before the
        batch is built). ``reflect`` (default on) asks every slice's plan for
        the reflection about the x axis where its scan allows it: many slices
        fill the GPU together, so the batch gains what a single small scan
        would not.
        ``fan_parts`` (1, 4, 16) sets the parts per walked ray of every turn
        slice's plan first (``Plan.set_tuning("fan_parts", ...)``)."""
        L = _lib.load()
        self.plans = [Plan(p) for p in paras]
        for i, P in enumerate(self.plans):
            if P.cone:
                raise ValueError(f"slice {i} is not a fan-beam scan")
            P.reflect = reflect and turns
            if not turns:
                P.rot_mirror = False
            if fan_parts is not None:
                P.set_tuning("fan_parts", fan_parts)
        # rays served per walk of each slice: 8 (quarter turns and the
        # reflection), 4 (quarter turns, or the half turn and the reflection),
        # 2 (half turn, or the reflection alone), 1
        self.turns = [P.views_per_walk for P in self.plans]
        self.reflect = [P.reflect for P in self.plans]
        n = len(self.plans)
        handles = (C.c_void_p * n)(*[P.handle.value for P in self.plans])
        h = C.c_void_p()
        _lib.check(L.fl_batch_create(handles, n, C.byref(h)))
        self._h, self._L = h, L
        vo = np.zeros(n + 1, np.int64)
        ro = np.zeros(n + 1, np.int64)
        _lib.check(L.fl_batch_layout(h, vo.ctypes.data, ro.ctypes.data))
        self.vox_offsets, self.ray_offsets = vo, ro
        self.n_vox, self.n_rays = int(vo[-1]), int(ro[-1])
        self.history = None
        self.iters_done = None

    def __len__(self):
        return len(self.plans)

    def autotune(self) -> int:
        """Times the parts per walked ray of the turn slices (1, 4, 16) on this
        batch's forward and keeps the fastest for all of them
        (``fl_batch_autotune``); returns it (0 without turn slices). The
        batch's forward then equals its plans' with that count set."""
        v = C.c_int32()
        _lib.check(self._L.fl_batch_autotune(self._h, _stream(), C.byref(v)))
        return v.value

    @property
    def launches_per_iteration(self) -> int:
        """Kernel launches of one CGLS iteration: forward and adjoint for each
        kind of slice present (general, turn, reflection), the transposed
        copy of the direction the forwards read, and the three algebra
        kernels."""
        general = any(t == 1 for t in self.turns)
        turned = any(t > 1 and not r for t, r in zip(self.turns, self.reflect))
        mirrored = any(self.reflect)
        return 4 + 2 * (int(general) + int(turned) + int(mirrored))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.fl_batch_destroy(h)
            self._h = None

    def _dev(self, t: torch.Tensor, n: int, what: str):
        if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and t.numel() == n):
            raise ValueError(f"{what}: expected a contiguous float32 CUDA tensor of {n} elements")

    def images(self, x: torch.Tensor):
        """Per-slice (ny, nx) views of a concatenated image tensor."""
        o = self.vox_offsets
        return [x[o[i]:o[i + 1]].view(P.ny, P.nx) for i, P in enumerate(self.plans)]

    def sinograms(self, y: torch.Tensor):
        """Per-slice (nv, nd) views of a concatenated sinogram tensor."""
        o = self.ray_offsets
        return [y[o[i]:o[i + 1]].view(P.nv, P.na) for i, P in enumerate(self.plans)]

    def concat_images(self, xs) -> torch.Tensor:
        return torch.cat([torch.as_tensor(x, dtype=torch.float32).reshape(-1) for x in xs])

    def forward(self, x: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        self._dev(x, self.n_vox, "forward input")
        y = torch.empty(self.n_rays, dtype=torch.float32, device=x.device) if out is None else out
        _lib.check(self._L.fl_batch_forward(self._h, x.data_ptr(), y.data_ptr(), _stream()))
        return y

    def adjoint(self, y: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        self._dev(y, self.n_rays, "adjoint input")
        x = torch.empty(self.n_vox, dtype=torch.float32, device=y.device) if out is None else out
        _lib.check(self._L.fl_batch_adjoint(self._h, y.data_ptr(), x.data_ptr(), _stream()))
        return x

    def cgls(self, rhs: torch.Tensor, u0: torch.Tensor | None = None, lam: float = 0.0,
             iters: int = 30, tol: float = 0.0) -> torch.Tensor:
        """Per-slice CGLS on (A_i^T A_i + lam I) u_i = rhs_i; ``history`` is then an
        (n_slices, iters) array of gamma_i after each iteration."""
        self._dev(rhs, self.n_vox, "right-hand side")
        if u0 is None:
            u, flags = torch.zeros_like(rhs), ZERO_START
        else:
            self._dev(u0, self.n_vox, "initial guess")
            u, flags = u0.clone(), 0
        n = len(self.plans)
        hist = np.zeros((n, max(iters, 1)), np.float64)
        done = np.zeros(n, np.int32)
        st = self._L.fl_batch_cgls(self._h, rhs.data_ptr(), u.data_ptr(), float(lam), int(iters),
                                   float(tol), flags, hist.ctypes.data, done.ctypes.data,
                                   _stream())
        self.history = hist[:, :iters]
        self.iters_done = done                # per slice, also when a slice stopped on NaN / Inf
        _lib.check(st)
        return u
