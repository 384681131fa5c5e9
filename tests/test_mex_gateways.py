"""The reference's own mex gateways, unmodified, against this library.

oracle/Makefile (target ``gateways``) compiles FrameLab's four gateways --
Ax_fan_mf.cpp, Atx_fan_mf.cpp, Ax_cone_mf.cpp, Atx_cone_mf.cpp -- from the
reference checkout with a stand-in for the mx API (oracle/mex/) and links
them as a mex build would: the GPU entry points they call (Ax_*_gpu_*,
Atx_*_gpu_*) resolve to libframelab_gb300.so, the CPU ones to the reference's
CPU kernels. Each golden fixture's ``para`` struct (MATLAB field names and
classes, as setPara.m builds them) then drives the gateway's own field
reading and dispatch (Ax_cone_mf.cpp:28-74 etc.):

* GPU = 0 runs the reference's CPU kernel through the gateway: the fixture
  must come back bit for bit (this checks the harness and the para structs);
* GPU = 1 runs this library's drop-in through the gateway: on a machine with
  a GPU it must give the same bits (the drop-ins are bit-exact replicas);
  without one, the call must reach the library, which reports that no CUDA
  device is present, instead of failing to link or crashing.

The gateways are built only where the reference sources exist (this file
skips elsewhere).
"""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from tests.golden.fixtures import load_case

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "oracle", "_ref")
GOLDEN = os.path.join(HERE, "golden")

CLASS = {np.dtype(np.float32): 7, np.dtype(np.float64): 6, np.dtype(np.int32): 12,
         np.dtype(np.uint32): 13}
# fixture kind -> (gateway, version, number of outputs)
KINDS = {"fan_siddon": ("Ax_fan_mf", 0, 1), "fan_new": ("Ax_fan_mf", 1, 1),
         "fan_fb": ("Ax_fan_mf", 2, 1), "fan_adj": ("Atx_fan_mf", 1, 1),
         "fan_fb_adj": ("Atx_fan_mf", 2, 1), "cone_siddon": ("Ax_cone_mf", 0, 1),
         "cone_new": ("Ax_cone_mf", 1, 2), "cone_adj": ("Atx_cone_mf", 1, 1)}


def _gateway(name):
    path = os.path.join(REF, f"mex_{name}.so")
    if not os.path.exists(path):
        pytest.skip("gateways not built here (reference sources absent)")
    g = C.CDLL(path)
    g.mh_numeric.restype = C.c_void_p
    g.mh_numeric.argtypes = [C.c_int, C.c_size_t, C.c_void_p]
    g.mh_struct.restype = C.c_void_p
    g.mh_set_field.argtypes = [C.c_void_p, C.c_char_p, C.c_void_p]
    g.mh_free.argtypes = [C.c_void_p]
    g.mxGetData.restype = C.c_void_p
    g.mxGetData.argtypes = [C.c_void_p]
    g.mxGetNumberOfElements.restype = C.c_size_t
    g.mxGetNumberOfElements.argtypes = [C.c_void_p]
    g.mexFunction.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p]
    return g


def _numeric(g, a):
    a = np.ascontiguousarray(np.asarray(a).reshape(-1, order="F"))
    return g.mh_numeric(CLASS[a.dtype], a.size, a.ctypes.data)


def _call(g, x, para, version, gpu, nout):
    para = dict(para, version=np.uint32(version), GPU=np.uint32(gpu))
    s = g.mh_struct()
    for k, v in para.items():
        v = np.asarray(v)
        if v.dtype in CLASS:
            g.mh_set_field(s, k.encode(), _numeric(g, v))
    prhs = (C.c_void_p * 2)(_numeric(g, np.asarray(x, np.float32)), s)
    plhs = (C.c_void_p * 2)()
    g.mexFunction(nout, plhs, 2, prhs)
    outs = []
    for k in range(nout):
        n = g.mxGetNumberOfElements(plhs[k])
        buf = (C.c_float * n).from_address(g.mxGetData(plhs[k]))
        outs.append(np.frombuffer(buf, np.float32).copy())
        g.mh_free(plhs[k])
    g.mh_free(prhs[0])
    g.mh_free(prhs[1])
    return outs


def _cases():
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        c = load_case(f)
        if c["kind"] in KINDS:
            out.append(pytest.param(f, id=os.path.basename(f)[:-4]))
    return out


def _has_cuda():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.parametrize("path", _cases())
def test_gateway_cpu_path_reproduces_fixture(path):
    c = load_case(path)
    name, version, nout = KINDS[c["kind"]]
    g = _gateway(name)
    outs = _call(g, c["x"], c["para"], version, 0, nout)
    assert np.array_equal(outs[0], c["y"])
    if nout == 2:
        assert np.array_equal(outs[1], c["extra"]["yNorm"])


@pytest.mark.parametrize("path", _cases())
def test_gateway_gpu_path_reaches_the_library(path):
    from framelab_gb300 import _lib
    c = load_case(path)
    name, version, nout = KINDS[c["kind"]]
    g = _gateway(name)
    L = _lib.load()
    outs = _call(g, c["x"], c["para"], version, 1, nout)
    if _has_cuda():
        assert L.fl_last_status() == _lib.FL_OK, L.fl_last_error()
        assert np.array_equal(outs[0], c["y"])
        if nout == 2:
            assert np.array_equal(outs[1], c["extra"]["yNorm"])
    else:
        # the drop-in ran and recorded the missing device
        assert L.fl_last_status() == _lib.FL_ERR_CUDA, L.fl_last_error()
