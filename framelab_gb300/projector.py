"""Projector plans over the C ABI (device tensors, CUDA streams).

A :class:`Plan` uploads one scan geometry (the reference's ``para`` struct) to
HBM once; ``forward``/``adjoint`` then run on device tensors on the current
PyTorch CUDA stream. Models:

* ``"siddon_ref"`` -- version 0, bit-exact with ``Ax_*_mf_cpu_siddon``
* ``"chord_ref"``  -- version 1 backprojector, bit-exact with ``Atx_*_mf_cpu_new``
* ``"gao_ref"``    -- version 1 forward, bit-exact with ``Ax_*_mf_cpu_new``
* ``"fb_ref"``     -- version 2 fan pair (finite-size beam), bit-exact with
  ``Ax_fan_mf_cpu_new_fb`` / ``Atx_fan_mf_cpu_new_fb``
* ``"matched"``    -- matched Siddon pair; the adjoint is the exact transpose
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib

MODELS = {"siddon_ref": _lib.MODEL_SIDDON_REF, "chord_ref": _lib.MODEL_CHORD_REF,
          "gao_ref": _lib.MODEL_GAO_REF, "fb_ref": _lib.MODEL_FB_REF,
          "matched": _lib.MODEL_MATCHED}
DTYPES = {torch.float32: _lib.F32, torch.float16: _lib.F16, torch.bfloat16: _lib.BF16}


def _arr(v, dt):
    return np.ascontiguousarray(np.asarray(v).reshape(-1).astype(dt))


def _stream(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


class Plan:
    """Geometry of one scan resident on the GPU."""

    def __init__(self, para: dict):
        L = _lib.load()
        self.para = para
        cone = "nz" in para
        self.cone = cone
        self.nx, self.ny = int(para["nx"]), int(para["ny"])
        self.nz = int(para["nz"]) if cone else 1
        self.nt = int(para.get("nt", 1))
        keep = {}

        def ptr(name, dt=np.float32):
            if name not in para or para[name] is None:
                return None
            a = _arr(para[name], dt)
            keep[name] = a
            return a.ctypes.data

        s = _lib.Scan()
        s.ndim = 3 if cone else 2
        s.nx, s.ny, s.nz, s.nt = self.nx, self.ny, self.nz, self.nt
        s.nv = len(np.asarray(para["sd_phi"]).reshape(-1))
        s.na = len(np.asarray(para["y_det"]).reshape(-1))
        s.nb = len(np.asarray(para["z_det"]).reshape(-1)) if cone else 1
        s.SO, s.OD, s.scale = float(para["SO"]), float(para["OD"]), float(para["scale"])
        s.dz = float(para["dz"]) if cone else 1.0
        s.dy_det = float(para.get("dy_det", 0.0))
        s.dz_det = float(para.get("dz_det", 0.0))
        s.y_os = float(para.get("y_os", 0.0))
        s.sd_phi = ptr("sd_phi")
        s.sd_z = ptr("sd_z") if cone else None
        s.y_det = ptr("y_det")
        s.z_det = ptr("z_det") if cone else None
        s.cos_phi, s.sin_phi = ptr("cos_phi"), ptr("sin_phi")
        if not cone:
            s.cos_det, s.sin_det = ptr("cos_det"), ptr("sin_det")
            s.cos_det2, s.sin_det2 = ptr("cos_det2"), ptr("sin_det2")
        s.view_frame = ptr("id_X", np.int32)
        if "id_Y" in para and "Nv" in para:
            idY = np.asarray(para["id_Y"])
            if idY.ndim == 2:          # MATLAB layout (tmp_size, nt), column-major
                idY = idY.T
            a = _arr(idY, np.int32)
            keep["id_Y"] = a
            s.id_Y = a.ctypes.data
            s.Nv = ptr("Nv", np.int32)
            s.tmp_size = int(para.get("tmp_size", a.size // max(self.nt, 1)))
        self.nv, self.na, self.nb = s.nv, s.na, s.nb
        h = C.c_void_p()
        _lib.check(L.fl_plan_create(C.byref(s), C.byref(h)))
        self._h = h
        self._L = L
        nv_, nr_ = C.c_int64(), C.c_int64()
        _lib.check(L.fl_plan_sizes(h, C.byref(nv_), C.byref(nr_)))
        self.n_vox, self.n_rays = nv_.value, nr_.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.fl_plan_destroy(h)
            self._h = None

    @property
    def z_mirror(self) -> bool:
        """Whether the matched pair uses the source-plane mirror symmetry
        (FL_OPT_Z_MIRROR; on by default where the scan allows it)."""
        v = C.c_int()
        _lib.check(self._L.fl_plan_query(self._h, _lib.OPT_Z_MIRROR, C.byref(v)))
        return bool(v.value)

    @z_mirror.setter
    def z_mirror(self, on: bool):
        _lib.check(self._L.fl_plan_option(self._h, _lib.OPT_Z_MIRROR, int(bool(on))))

    @property
    def rot_mirror(self) -> bool:
        """Whether the matched pair also uses the half-turn symmetry between
        views v and v + nv/2 (FL_OPT_ROT_MIRROR; a cone plan needs the z
        mirror for it, a fan plan an even ny)."""
        v = C.c_int()
        _lib.check(self._L.fl_plan_query(self._h, _lib.OPT_ROT_MIRROR, C.byref(v)))
        return bool(v.value)

    @rot_mirror.setter
    def rot_mirror(self, on: bool):
        _lib.check(self._L.fl_plan_option(self._h, _lib.OPT_ROT_MIRROR, int(bool(on))))

    @property
    def quarter_turn(self) -> bool:
        """Whether the matched pair also uses the quarter-turn symmetry between
        views v and v + nv/4 (FL_OPT_QUARTER_TURN; needs the half turn)."""
        v = C.c_int()
        _lib.check(self._L.fl_plan_query(self._h, _lib.OPT_QUARTER_TURN, C.byref(v)))
        return bool(v.value)

    @quarter_turn.setter
    def quarter_turn(self, on: bool):
        _lib.check(self._L.fl_plan_option(self._h, _lib.OPT_QUARTER_TURN, int(bool(on))))

    @property
    def reflect(self) -> bool:
        """Whether the matched pair also uses the reflection between views v
        and nv - v about the x axis (FL_OPT_REFLECT; with the half or the
        quarter turn and a detector symmetric about its centre, or, on a fan
        plan of an odd view count, alone). On by default for cone plans; fan
        plans take it when it is set (FanBatch sets it for its slices)."""
        v = C.c_int()
        _lib.check(self._L.fl_plan_query(self._h, _lib.OPT_REFLECT, C.byref(v)))
        return bool(v.value)

    @reflect.setter
    def reflect(self, on: bool):
        _lib.check(self._L.fl_plan_option(self._h, _lib.OPT_REFLECT, int(bool(on))))

    @property
    def rotations(self) -> int:
        """Turns of the matched kernels in use: 4 (quarter turns), 2 (half
        turn) or 1."""
        if self.quarter_turn:
            return 4
        return 2 if self.rot_mirror else 1

    @property
    def views_per_walk(self) -> int:
        """Views one walk or weight of the matched kernels in use serves: the
        rotations, twice that with the reflection (8, 4, 2 or 1)."""
        return self.rotations * (2 if self.reflect else 1)

    # launch variants fl_plan_autotune chooses among (fl_plan_option values)
    TUNABLES = {"adj_run": _lib.TUNE_ADJ_RUN, "adj_rows": _lib.TUNE_ADJ_ROWS,
                "fan_parts": _lib.TUNE_FAN_PARTS, "fan_block": _lib.TUNE_FAN_BLOCK,
                "fan_groups": _lib.TUNE_FAN_GROUPS, "adj_chunks": _lib.TUNE_ADJ_CHUNKS,
                "fan_tma": _lib.TUNE_FAN_TMA}

    def tuning(self, name: str) -> int:
        """The value in effect of a launch variant (``TUNABLES``)."""
        v = C.c_int()
        _lib.check(self._L.fl_plan_query(self._h, self.TUNABLES[name], C.byref(v)))
        return v.value

    def set_tuning(self, name: str, value: int):
        """Sets a launch variant (``TUNABLES``); values outside its set raise."""
        _lib.check(self._L.fl_plan_option(self._h, self.TUNABLES[name], int(value)))

    @property
    def handle(self):
        return self._h

    @property
    def vol_shape(self):
        return (self.nt, self.nz, self.ny, self.nx) if self.cone else (self.nt, self.ny, self.nx)

    @property
    def sino_shape(self):
        return (self.nv, self.nb, self.na) if self.cone else (self.nv, self.na)

    def _check_dev(self, t, n, what):
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.is_contiguous()):
            raise ValueError(f"{what} must be a contiguous CUDA tensor")
        if t.numel() != n:
            raise ValueError(f"{what} has {t.numel()} elements, expected {n}")
        if t.dtype not in DTYPES:
            raise ValueError(f"{what}: unsupported dtype {t.dtype}")

    def forward(self, x: torch.Tensor, model: str = "matched", out: torch.Tensor | None = None,
                out_dtype=None, stream=None) -> torch.Tensor:
        self._check_dev(x, self.n_vox, "x")
        if out is None:
            out = torch.empty(self.sino_shape, device=x.device,
                              dtype=out_dtype or torch.float32)
        self._check_dev(out, self.n_rays, "out")
        _lib.check(self._L.fl_forward(self._h, MODELS[model], x.data_ptr(), DTYPES[x.dtype],
                                      out.data_ptr(), DTYPES[out.dtype], _stream(stream)))
        return out

    def adjoint(self, y: torch.Tensor, model: str = "matched", out: torch.Tensor | None = None,
                out_dtype=None, stream=None) -> torch.Tensor:
        self._check_dev(y, self.n_rays, "y")
        if out is None:
            out = torch.empty(self.vol_shape, device=y.device, dtype=out_dtype or torch.float32)
        self._check_dev(out, self.n_vox, "out")
        _lib.check(self._L.fl_adjoint(self._h, MODELS[model], y.data_ptr(), DTYPES[y.dtype],
                                      out.data_ptr(), DTYPES[out.dtype], _stream(stream)))
        return out

    def forward_gao(self, x: torch.Tensor, with_norm: bool = True, stream=None):
        """Version-1 forward (Ax_*_mf_cpu_new); cone beams also return yNorm."""
        self._check_dev(x, self.n_vox, "x")
        if x.dtype != torch.float32:
            raise ValueError("version-1 forward is FP32 only")
        y = torch.empty(self.sino_shape, device=x.device, dtype=torch.float32)
        yn = torch.empty_like(y) if (with_norm and self.cone) else None
        _lib.check(self._L.fl_forward_gao(self._h, x.data_ptr(), y.data_ptr(),
                                          yn.data_ptr() if yn is not None else None,
                                          _stream(stream)))
        return (y, yn) if yn is not None else y

    def autotune(self, stream=None) -> dict:
        """Times the launch variants of this plan's matched projector kernels
        on its own geometry and keeps the fastest (``fl_plan_autotune``).
        Cone plans: the block shapes (and, on a reflection plan, the
        backprojection's voxels per thread and row loop); the projections do
        not change. Fan plans: the parts per walked ray of the turn forward
        (the order of a ray's additions) and the backprojection's pixel block
        (the same bits). Plans without a matched backprojection report
        ``None``."""
        sh = (C.c_int32 * 4)()
        _lib.check(self._L.fl_plan_autotune(self._h, _stream(stream), sh))
        if not sh[0]:
            return {"forward": None, "adjoint": None}
        if not self.cone:
            return {"forward_parts_per_ray": sh[0], "adjoint_pixel_block": sh[2],
                    "adjoint_view_groups": sh[3]}
        out = {"forward": (sh[0], sh[1]), "adjoint": (sh[2], sh[3])}
        if self.reflect:
            v = C.c_int()
            _lib.check(self._L.fl_plan_query(self._h, _lib.TUNE_ADJ_RUN, C.byref(v)))
            out["adjoint_voxels_per_thread"] = v.value
            _lib.check(self._L.fl_plan_query(self._h, _lib.TUNE_ADJ_ROWS, C.byref(v)))
            out["adjoint_rows_per_iteration"] = v.value
            _lib.check(self._L.fl_plan_query(self._h, _lib.TUNE_ADJ_CHUNKS, C.byref(v)))
            out["adjoint_view_chunks"] = v.value
        return out

    def count_intersections(self, stream=None) -> torch.Tensor:
        c = torch.empty(self.sino_shape, device="cuda", dtype=torch.int32)
        _lib.check(self._L.fl_count_intersections(self._h, c.data_ptr(), _stream(stream)))
        return c
