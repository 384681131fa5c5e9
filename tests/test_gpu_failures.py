"""Failure paths without a GPU fault: every device allocation of the library
can be made to fail (fl_debug_fail_alloc). Walking the failure point through
plan creation, CGLS workspaces, solves, framelets, split Bregman and a batch
gives clean FL_ERR_ALLOC errors, leaks no device memory, and leaves the
library working with the same results as before."""
import gc

import numpy as np
import pytest

from framelab_gb300 import geometry as G
from framelab_gb300 import phantoms as PH

pytestmark = pytest.mark.gpu


def _workload(p, x, f, fan):
    import torch
    from framelab_gb300.batch import FanBatch
    from framelab_gb300.projector import Plan
    from framelab_gb300.solvers import NativeCGLS
    from framelab_gb300.transforms import split_bregman
    P = Plan(p)
    y = P.forward(x)
    b = P.adjoint(y).reshape(-1)
    u = NativeCGLS(P, "graph").solve(b, iters=3)
    um = NativeCGLS(P, "mixed").solve(b, iters=3, refresh=2)
    s, _ = split_bregman(P, f, torch.zeros_like(u), lam=0.01, mu=1.0, outer=1, cg_iters=2,
                         levels=1)
    B = FanBatch([fan])
    ub = B.cgls(B.adjoint(B.forward(torch.ones(B.n_vox, device="cuda"))), iters=2)
    torch.cuda.synchronize()
    return [t.detach().cpu().numpy().copy() for t in (y, u, um, s, ub)]


def test_allocation_failures_are_clean_errors():
    import torch
    from framelab_gb300 import _lib
    L = _lib.load()
    p = G.cone_para_mm(24, 12, 36, 28, det_pitch_mm=8.0, SO_mm=600.0, SD_mm=1200.0,
                       voxel_mm=8.0)
    fan = G.fan_para(32, 32, 48, 10, L=(1, 1))
    x = torch.from_numpy(PH.ellipsoids_3d(24, seed=1).reshape(-1)).cuda()
    from framelab_gb300.projector import Plan
    f = Plan(p).forward(x)
    ref = _workload(p, x, f, fan)               # also creates the persistent dot scratch
    gc.collect()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    outcomes = []
    for nth in range(1, 400):
        L.fl_debug_fail_alloc(nth)
        try:
            _workload(p, x, f, fan)
            outcomes.append("ok")
        except _lib.FLError as e:
            assert e.code == _lib.FL_ERR_ALLOC, (nth, str(e))
            outcomes.append("alloc")
        finally:
            L.fl_debug_fail_alloc(0)
        if outcomes[-1] == "ok":
            break
    assert outcomes.count("alloc") >= 20 and outcomes[-1] == "ok", outcomes
    gc.collect()
    torch.cuda.synchronize()
    leaked = free0 - torch.cuda.mem_get_info()[0]
    assert leaked < 32 << 20, f"{leaked} bytes of device memory not released"
    again = _workload(p, x, f, fan)
    for a, r in zip(again, ref):
        assert np.array_equal(a, r)


@pytest.mark.parametrize("mode", ["plain", "graph", "mixed"])
def test_nonfinite_rhs_stops_with_numeric_error(mode):
    import torch
    from framelab_gb300 import _lib
    from framelab_gb300.projector import Plan
    from framelab_gb300.solvers import NativeCGLS
    p = G.cone_para_mm(24, 12, 36, 28, det_pitch_mm=8.0, SO_mm=600.0, SD_mm=1200.0,
                       voxel_mm=8.0)
    P = Plan(p)
    x = torch.from_numpy(PH.ellipsoids_3d(24, seed=2).reshape(-1)).cuda()
    b = P.adjoint(P.forward(x)).reshape(-1).contiguous()
    cg = NativeCGLS(P, mode)
    want = cg.solve(b, iters=4).clone()
    bad = b.clone()
    bad[1234] = float("nan")
    with pytest.raises(_lib.FLError) as e:
        cg.solve(bad, iters=4)
    assert e.value.code == _lib.FL_ERR_NUMERIC
    assert cg.iters_done == 0
    # the workspace is still good: the same solve gives the same bits
    assert torch.equal(cg.solve(b, iters=4), want)


@pytest.mark.parametrize("mode", ["plain", "graph", "mixed"])
def test_zero_rhs_returns_the_start_without_iterating(mode):
    import torch
    from framelab_gb300.projector import Plan
    from framelab_gb300.solvers import NativeCGLS
    p = G.cone_para_mm(16, 8, 24, 20, det_pitch_mm=8.0, SO_mm=600.0, SD_mm=1200.0,
                       voxel_mm=8.0)
    P = Plan(p)
    cg = NativeCGLS(P, mode)
    u = cg.solve(torch.zeros(P.n_vox, device="cuda"), iters=5)
    assert cg.iters_done == 0
    assert bool(torch.all(u == 0))


def test_batch_nonfinite_slice_is_reported_and_others_complete():
    import torch
    from framelab_gb300 import _lib
    from framelab_gb300.batch import FanBatch
    paras = [G.fan_para(n, n, 2 * n, v, L=(1, 1)) for n, v in ((24, 9), (32, 12), (20, 7))]
    B = FanBatch(paras)
    rhs = B.adjoint(B.forward(torch.ones(B.n_vox, device="cuda")))
    good = B.cgls(rhs, iters=4).clone()
    bad = rhs.clone()
    B.images(bad)[1][3, 4] = float("inf")
    with pytest.raises(_lib.FLError) as e:
        B.cgls(bad, iters=4)
    assert e.value.code == _lib.FL_ERR_NUMERIC and "slice 1" in str(e.value)
    assert list(B.iters_done) == [4, 0, 4]      # the other slices ran to the end
    assert torch.equal(B.cgls(rhs, iters=4), good)


def test_tma_wait_that_runs_out_is_reported_and_the_context_stays_usable():
    """The fan forward's TMA copy waits on an mbarrier for a bounded number of
    polls. FL_DEBUG_TMA_STALL makes that wait run out with nothing in flight
    (no load is issued; the phase it waits on is never completed): the plan's
    flag reads 1 once and is then cleared, a solve whose forwards timed out
    returns FL_ERR_TIMEOUT, and with the hook off the same plan and context
    give the same bits as before."""
    import ctypes as C
    import torch
    from framelab_gb300 import _lib
    from framelab_gb300.projector import Plan
    from framelab_gb300.solvers import NativeCGLS
    L = _lib.load()
    P = Plan(G.fan_para(64, 64, 128, 20, L=(1, 1), SO=3.0, OD=3.0, Ly=3.0))
    assert P.tuning("fan_tma") == 1
    x = torch.from_numpy(PH.ellipses_2d(64, seed=3).reshape(-1)).cuda()
    y = P.forward(x).clone()
    b = P.adjoint(y).reshape(-1).contiguous()
    want = NativeCGLS(P, "plain").solve(b, iters=3).clone()

    def flag():
        v = C.c_int(-1)
        _lib.check(L.fl_plan_query(P.handle, _lib.DEBUG_TMA_TIMEOUTS, C.byref(v)))
        return v.value

    assert flag() == 0
    assert L.fl_plan_option(P.handle, _lib.DEBUG_TMA_STALL, -1) == _lib.FL_ERR_INVALID
    _lib.check(L.fl_plan_option(P.handle, _lib.DEBUG_TMA_STALL, 1000))
    P.forward(x)
    torch.cuda.synchronize()
    assert flag() == 1 and flag() == 0            # read once, then cleared
    cg = NativeCGLS(P, "plain")
    with pytest.raises(_lib.FLError) as e:
        cg.solve(b, iters=3)
    assert e.value.code == _lib.FL_ERR_TIMEOUT
    assert flag() == 0
    _lib.check(L.fl_plan_option(P.handle, _lib.DEBUG_TMA_STALL, 0))
    assert torch.equal(P.forward(x), y)
    assert torch.equal(NativeCGLS(P, "plain").solve(b, iters=3), want)
    assert flag() == 0
