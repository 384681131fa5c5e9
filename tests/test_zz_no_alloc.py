"""fl_adjoint_noalloc: the matched backprojection without device allocation.

Callers that cannot allocate device memory when they backproject (a CUDA graph
being captured, an application whose pool allocator owns the GPU memory) use
this entry point; its scratch is a fixed array inside the library. Checked
through the C ABI against fl_adjoint, on two calls in a row with different
inputs (the shared scratch keeps the previous call's contents), and for the
refusal of plans larger than the fixed scratch. This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from framelab_gb300 import _lib
from framelab_gb300 import geometry as G

pytestmark = pytest.mark.gpu

MAX_RAYS = 1 << 21


def _entry():
    L = _lib.load()
    _lib.declare("fl_adjoint_noalloc", C.c_int,
                 [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p])
    return L


@pytest.mark.parametrize("which", ["fan", "cone"])
def test_noalloc_adjoint_matches_fl_adjoint_on_two_calls(which):
    import torch
    from framelab_gb300.projector import Plan
    L = _entry()
    if which == "fan":
        para = G.fan_para(96, 96, 192, 180, L=(1.0, 1.0), SO=3.0, OD=3.0, Ly=3.0)
    else:
        para = G.cone_para_mm(32, 24, 48, 40, det_pitch_mm=8.0, SO_mm=600.0, SD_mm=1200.0,
                              voxel_mm=8.0)
    P = Plan(para)
    assert P.n_rays <= MAX_RAYS
    g = torch.Generator(device="cuda").manual_seed(7)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        y = torch.randn(P.sino_shape, device="cuda", generator=g) * (1.0 + call)
        want = P.adjoint(y)                       # fl_adjoint (plan-owned scratch)
        got = torch.full(P.vol_shape, float("nan"), device="cuda")
        st = L.fl_adjoint_noalloc(P.handle, y.data_ptr(), _lib.F32, got.data_ptr(), _lib.F32,
                                  stream)
        assert st == _lib.FL_OK, L.fl_last_error()
        torch.cuda.synchronize()
        err = (got - want).abs().max().item()
        assert err <= 1e-6 * want.abs().max().item(), (call, err)


def test_noalloc_adjoint_refuses_plans_beyond_its_scratch():
    import torch
    from framelab_gb300.projector import Plan
    L = _entry()
    para = G.fan_para(16, 16, MAX_RAYS + 2, 1, L=(1.0, 1.0), SO=40.0, OD=40.0, Ly=60.0)
    P = Plan(para)
    assert P.n_rays > MAX_RAYS
    y = torch.zeros(P.n_rays, device="cuda")
    x = torch.zeros(P.n_vox, device="cuda")
    st = L.fl_adjoint_noalloc(P.handle, y.data_ptr(), _lib.F32, x.data_ptr(), _lib.F32,
                              torch.cuda.current_stream().cuda_stream)
    assert st == _lib.FL_ERR_INVALID
    assert b"exceed" in L.fl_last_error()
