"""ctypes binding of libframelab_gb300.so (the C ABI in include/framelab_gb300.h).

The library is the only compute path: if it cannot be loaded, every operator
raises. There is no CPU or PyTorch fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

(FL_OK, FL_ERR_INVALID, FL_ERR_UNSUPPORTED, FL_ERR_CUDA, FL_ERR_ALLOC, FL_ERR_TIMEOUT,
 FL_ERR_NUMERIC) = range(7)
MODEL_SIDDON_REF, MODEL_CHORD_REF, MODEL_GAO_REF, MODEL_FB_REF, MODEL_MATCHED = 0, 1, 2, 3, 16
F32, F16, BF16 = 0, 1, 2
OPT_Z_MIRROR = 1
OPT_ROT_MIRROR = 2
OPT_QUARTER_TURN = 3
OPT_REFLECT = 4
TUNE_ADJ_RUN = 16
TUNE_ADJ_ROWS = 17
TUNE_FAN_PARTS = 18
TUNE_FAN_BLOCK = 19
TUNE_FAN_GROUPS = 20
TUNE_ADJ_CHUNKS = 21
TUNE_FAN_TMA = 22
DEBUG_TMA_TIMEOUTS = 23
DEBUG_TMA_STALL = 24
FRAMELET_OPT_FUSED = 1


class FLError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"framelab_gb300 error {code}: {msg}")
        self.code = code


class Scan(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("nt", C.c_int32), ("nv", C.c_int32), ("na", C.c_int32), ("nb", C.c_int32),
        ("SO", C.c_float), ("OD", C.c_float), ("scale", C.c_float), ("dz", C.c_float),
        ("dy_det", C.c_float), ("dz_det", C.c_float), ("y_os", C.c_float),
        ("sd_phi", C.c_void_p), ("sd_z", C.c_void_p), ("y_det", C.c_void_p),
        ("z_det", C.c_void_p), ("cos_phi", C.c_void_p), ("sin_phi", C.c_void_p),
        ("cos_det", C.c_void_p), ("sin_det", C.c_void_p), ("view_frame", C.c_void_p),
        ("id_Y", C.c_void_p), ("Nv", C.c_void_p), ("tmp_size", C.c_int32),
        ("cos_det2", C.c_void_p), ("sin_det2", C.c_void_p),
    ]


_V, _I, _I64, _F, _D = C.c_void_p, C.c_int, C.c_int64, C.c_float, C.c_double
_P = C.c_void_p

# name -> (restype, argtypes)
_SIGS = {
    "fl_last_status": (_I, []),
    "fl_last_error": (C.c_char_p, []),
    "fl_version": (C.c_char_p, []),
    "fl_plan_create": (_I, [C.POINTER(Scan), C.POINTER(_P)]),
    "fl_plan_destroy": (None, [_P]),
    "fl_plan_sizes": (_I, [_P, C.POINTER(_I64), C.POINTER(_I64)]),
    "fl_plan_option": (_I, [_P, _I, _I]),
    "fl_plan_query": (_I, [_P, _I, C.POINTER(_I)]),
    "fl_plan_autotune": (_I, [_P, _P, _P]),
    "fl_forward": (_I, [_P, _I, _V, _I, _V, _I, _V]),
    "fl_adjoint": (_I, [_P, _I, _V, _I, _V, _I, _V]),
    "fl_count_intersections": (_I, [_P, _V, _V]),
    "fl_forward_gao": (_I, [_P, _V, _V, _V, _V]),
    "Ax_fan_mf_gpu_new": (None, [_V, _V, _F, _F, _F, _I, _I, _I, _V, _I, _V, _V, _I]),
    "Ax_cone_mf_gpu_new": (None, [_V, _V, _V, _V, _V, _V, _V, _V, _V, _F, _F, _F, _F, _I, _I,
                                  _I, _I, _I, _I, _I, _I, _I]),
    "Ax_fan_mf_gpu_siddon": (None, [_V, _V, _F, _F, _F, _I, _I, _I, _V, _I, _V, _V, _I]),
    "Atx_fan_mf_gpu_new": (None, [_V, _V, _F, _F, _F, _I, _I, _V, _I, _V, _F, _F, _I, _V, _V,
                                  _I, _I, _V, _V, _V, _V]),
    "Ax_fan_mf_gpu_new_fb": (None, [_V, _V, _F, _F, _F, _I, _I, _I, _V, _I, _V, _V, _I, _F]),
    "Atx_fan_mf_gpu_new_fb": (None, [_V, _V, _F, _F, _F, _I, _I, _V, _I, _V, _F, _I, _V, _V,
                                     _I, _I, _V, _V, _V, _V]),
    "Ax_cone_mf_gpu_siddon": (None, [_V, _V, _V, _V, _V, _V, _V, _V, _F, _F, _F, _F, _I, _I,
                                     _I, _I, _I, _I, _I, _I, _I]),
    "Atx_cone_mf_gpu_new": (None, [_V, _V, _V, _V, _V, _V, _V, _V, _V, _F, _F, _F, _F, _F, _F,
                                   _F, _I, _I, _I, _I, _I, _I, _I, _I, _I]),
    "fl_adjoint_noalloc": (_I, [_P, _V, _I, _V, _I, _V]),
    "fl_debug_bounds": (_I, [C.POINTER(_I64), _I]),
    "fl_debug_fail_alloc": (None, [_I64]),
    # vector algebra and CGLS
    "fl_dot": (_I, [_V, _V, _I64, _V, _V]),
    "fl_axpby": (_I, [_V, _V, _F, _F, _I64, _V]),
    "fl_normal_apply": (_I, [_P, _V, _V, _F, _V]),
    "fl_cgls_create": (_I, [_P, _I, C.POINTER(_P)]),
    "fl_cgls_destroy": (None, [_P]),
    "fl_cgls_solve": (_I, [_P, _V, _V, _F, _I, _D, _I, _I, _V, C.POINTER(_I), _V]),
    "fl_cgls_solve_host": (_I, [_P, _V, _V, _F, _I, _D, _I, _I, _V, C.POINTER(_I), _V]),
    # framelets and split Bregman
    "fl_framelet_create": (_I, [_I, _I, _I, _I, _I, C.POINTER(_P)]),
    "fl_framelet_destroy": (None, [_P]),
    "fl_framelet_ncoef": (_I64, [_P]),
    "fl_framelet_analysis": (_I, [_P, _V, _V, _V]),
    "fl_framelet_synthesis": (_I, [_P, _V, _V, _V]),
    "fl_framelet_bregman": (_I, [_P, _V, _V, _V, _V, _F, _F, _V, _V]),
    "fl_framelet_shrink": (_I, [_P, _V, _V, _F, _V]),
    "fl_framelet_option": (_I, [_P, _I, _I]),
    "fl_sb_solve": (_I, [_P, _V, _V, _F, _F, _I, _I, _D, _I, _I, _I, _V, _V]),
    "fl_sb_create": (_I, [_P, _I, _I, _I, C.POINTER(_P)]),
    "fl_sb_run": (_I, [_P, _V, _V, _F, _F, _I, _I, _D, _V, _V]),
    "fl_sb_destroy": (None, [_P]),
    # batched fan slices
    "fl_batch_create": (_I, [C.POINTER(_P), C.c_int32, C.POINTER(_P)]),
    "fl_batch_destroy": (None, [_P]),
    "fl_batch_layout": (_I, [_P, _V, _V]),
    "fl_batch_forward": (_I, [_P, _V, _V, _V]),
    "fl_batch_adjoint": (_I, [_P, _V, _V, _V]),
    "fl_batch_cgls": (_I, [_P, _V, _V, _F, C.c_int32, _D, C.c_int32, _V, _V, _V]),
    "fl_batch_autotune": (_I, [_P, _V, _V]),
}


class _Checked:
    """The loaded library. Only functions with a signature in _SIGS can be
    reached: a ctypes call without argtypes would pass 64-bit device
    pointers as 32-bit C ints."""

    def __init__(self, cdll):
        self._cdll = cdll

    def __getattr__(self, name):
        if name not in _SIGS:
            raise AttributeError(f"{name}: no signature registered in framelab_gb300._lib")
        return getattr(self._cdll, name)


# FRAMELAB_GB300_VARIANT selects a build variant of the library for this
# process ("checked": bounds-checked gathers, framelab_gb300.build.VARIANTS)
_VARIANT = os.environ.get("FRAMELAB_GB300_VARIANT", "")


def lib_path() -> str:
    return _build.variant_path(_VARIANT)


def load(build_if_missing: bool = True):
    """Load the library (building it in-tree first when it is absent)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.variant_path(_VARIANT)
            if build_if_missing:
                path = _build.build(variant=_VARIANT)
            if not os.path.exists(path):
                raise FLError(FL_ERR_CUDA, f"{path} not built; run framelab_gb300.build.build()")
            lib = C.CDLL(path)
            for name, (res, args) in _SIGS.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = _Checked(lib)
        return _lib


def declare(name, restype, argtypes):
    """Register the signature of an additional exported symbol."""
    _SIGS[name] = (restype, argtypes)
    if _lib is not None:
        fn = getattr(_lib._cdll, name)
        fn.restype = restype
        fn.argtypes = argtypes


def check(status: int):
    if status != FL_OK:
        L = load()
        raise FLError(status, L.fl_last_error().decode())


def check_last():
    L = load()
    check(L.fl_last_status())
