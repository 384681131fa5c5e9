"""fl_adjoint_noalloc: the matched backprojection without device allocation.

Some callers cannot allocate device memory when they backproject: work being
captured into a CUDA graph, a host application whose pool allocator owns the
GPU's memory, a loop that must not block on the allocator. This entry point
keeps its scratch in a fixed array inside the library instead of the plan.

Checked through the C ABI:
* on a fresh plan that has never run a backprojection, the no-alloc call runs
  first, with the library's allocation hook armed to fail the next device
  allocation and with the device's free memory recorded: it must succeed and
  leave the free memory unchanged (it allocates nothing);
* its results equal fl_adjoint's bit for bit (the same kernels, launch shapes
  and inputs), on two calls in a row, the second with a sinogram a thousand
  times smaller, so contents left in the shared scratch by the first call
  would show;
* plans larger than the fixed scratch are refused.
This file is collected last.
"""
import ctypes as C

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


def _para(which):
    if which == "fan":
        return G.fan_para(96, 96, 192, 180, L=(1.0, 1.0), SO=3.0, OD=3.0, Ly=3.0)
    return G.cone_para_mm(32, 24, 48, 40, det_pitch_mm=8.0, SO_mm=600.0, SD_mm=1200.0,
                          voxel_mm=8.0)


@pytest.mark.parametrize("which", ["fan", "cone"])
def test_noalloc_adjoint_matches_fl_adjoint_on_two_calls(which):
    import torch
    from framelab_gb300.projector import Plan
    L = _entry()
    stream = torch.cuda.current_stream().cuda_stream
    # the first call on this device places the library's fixed array on it;
    # make it on a plan of its own, as a user does at start-up
    P0 = Plan(_para(which))
    y0 = torch.zeros(P0.sino_shape, device="cuda")
    x0 = torch.empty(P0.vol_shape, device="cuda")
    assert L.fl_adjoint_noalloc(P0.handle, y0.data_ptr(), _lib.F32, x0.data_ptr(), _lib.F32,
                                stream) == _lib.FL_OK, L.fl_last_error()
    P = Plan(_para(which))
    assert P.n_rays <= MAX_RAYS
    g = torch.Generator(device="cuda").manual_seed(7)
    ys = [torch.randn(P.sino_shape, device="cuda", generator=g),
          1e-3 * torch.randn(P.sino_shape, device="cuda", generator=g)]
    got = [torch.full(P.vol_shape, float("nan"), device="cuda") for _ in ys]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for y, x in zip(ys, got):
        L.fl_debug_fail_alloc(1)                  # the next device allocation would fail
        try:
            st = L.fl_adjoint_noalloc(P.handle, y.data_ptr(), _lib.F32, x.data_ptr(),
                                      _lib.F32, stream)
        finally:
            L.fl_debug_fail_alloc(0)
        assert st == _lib.FL_OK, L.fl_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0   # nothing was allocated
    for y, x in zip(ys, got):
        want = P.adjoint(y)                       # fl_adjoint (plan-owned scratch)
        torch.cuda.synchronize()
        assert torch.equal(x, want)


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
