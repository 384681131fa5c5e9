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
