"""CGLS on the GPU against the FP64 restatement of solveCGLS.m (oracle/numerics.py)
driven by the FP64 exact projector pair (oracle)."""
import numpy as np
import pytest

import oracle as O
from oracle import numerics as N
from framelab_gb300 import geometry as G
from framelab_gb300 import phantoms as PH

pytestmark = pytest.mark.gpu


def _setup(n=24, nv=16):
    p = G.cone_para_mm(n, nv, 36, 32, det_pitch_mm=8.0, SO_mm=600.0, SD_mm=1200.0, voxel_mm=8.0)
    x = PH.ellipsoids_3d(n, seed=2).reshape(-1).astype(np.float64)
    f = O.exact_forward(x, p, threads=8)
    b = O.exact_adjoint(f, p, threads=8)
    return p, x, b


def _oracle_solution(p, b, lam, iters):
    normal = lambda v: O.exact_adjoint(O.exact_forward(v, p, threads=8), p, threads=8)  # noqa: E731
    return N.cgls(normal, b, np.zeros_like(b), lam, iters)


def test_dot_fp64():
    import torch
    from framelab_gb300.solvers import dot
    g = torch.Generator().manual_seed(0)
    a = torch.randn(1_000_003, generator=g)
    c = torch.randn(1_000_003, generator=g)
    want = float(np.dot(a.double().numpy(), c.double().numpy()))
    got = dot(a.cuda(), c.cuda())
    assert abs(got - want) <= 1e-12 * np.sqrt(a.numel()) * float(np.linalg.norm(a) * np.linalg.norm(c))


@pytest.mark.parametrize("mode", ["plain", "graph", "mixed"])
def test_cgls_matches_fp64_oracle(mode):
    import torch
    from framelab_gb300.projector import Plan
    from framelab_gb300.solvers import NativeCGLS
    p, x, b = _setup()
    lam, iters = 0.5, 12
    u64, h64 = _oracle_solution(p, b, lam, iters)
    P = Plan(p)
    cg = NativeCGLS(P, mode)
    u = cg.solve(torch.from_numpy(b.astype(np.float32)).cuda(), lam=lam, iters=iters,
                 refresh=5).cpu().numpy().reshape(-1)
    rel = np.linalg.norm(u - u64) / np.linalg.norm(u64)
    tol = 1e-3 if mode == "mixed" else 1e-4
    assert rel < tol, (mode, rel)
    assert cg.iters_done == iters
    g = np.array(cg.history)
    assert np.all(np.isfinite(g)) and g[-1] < g[0]


def test_cgls_early_stop_and_warm_start():
    import torch
    from framelab_gb300.projector import Plan
    from framelab_gb300.solvers import NativeCGLS
    p, x, b = _setup(16, 8)
    P = Plan(p)
    bt = torch.from_numpy(b.astype(np.float32)).cuda()
    cg = NativeCGLS(P, "mixed")
    u = cg.solve(bt, lam=1.0, iters=50, tol=1e30)   # stops after the first iteration
    assert cg.iters_done == 1
    cg2 = NativeCGLS(P, "plain")
    u1 = cg2.solve(bt, lam=1.0, iters=3)
    u2 = cg2.solve(bt, u0=u1, lam=1.0, iters=3, zero_start=False)
    u6 = cg2.solve(bt, lam=1.0, iters=6)
    r = lambda v: np.linalg.norm(v.cpu().numpy())  # noqa: E731
    assert r(u2 - u6) / r(u6) < 0.2     # warm restart lands near the 6-iteration solution


@pytest.mark.parametrize("mode", ["graph", "mixed"])
def test_cgls_z_folded_vectors_follow_the_plan_option(mode):
    """On a source-plane-symmetric scan the fused forms keep their vectors
    z-folded; turning the plan's mirror option off between solves on the same
    workspace switches to the general kernels and standard layout."""
    import torch
    from framelab_gb300.projector import Plan
    from framelab_gb300.solvers import NativeCGLS
    p, x, b = _setup(16, 8)
    P = Plan(p)
    assert P.z_mirror
    bt = torch.from_numpy(b.astype(np.float32)).cuda()
    cg = NativeCGLS(P, mode)
    u_m = cg.solve(bt, lam=0.5, iters=6, refresh=3)
    P.z_mirror = False
    u_g = cg.solve(bt, lam=0.5, iters=6, refresh=3)
    P.z_mirror = True
    u_m2 = cg.solve(bt, lam=0.5, iters=6, refresh=3)
    rel = float((u_m - u_g).norm() / u_g.norm())
    assert rel < (1e-3 if mode == "mixed" else 1e-5), rel
    assert torch.equal(u_m, u_m2)
    u64, _ = _oracle_solution(p, b, 0.5, 6)
    assert np.linalg.norm(u_m.cpu().numpy() - u64) / np.linalg.norm(u64) < 1e-3


@pytest.mark.parametrize("mode", ["plain", "graph", "mixed"])
def test_host_buffer_solve_equals_the_device_solve(mode):
    """fl_cgls_solve_host gives the device solve's bits, from pageable numpy
    buffers (staged copies) and from pinned ones (a z-mirror plan in the
    graph and mixed forms reads b and writes u in host memory directly), with
    a zero start and with a given u0 (read in place too)."""
    import torch
    from framelab_gb300.projector import Plan
    from framelab_gb300.solvers import NativeCGLS
    p = G.cone_para_mm(24, 20, 36, 28, det_pitch_mm=8.0, SO_mm=600.0, SD_mm=1200.0,
                       voxel_mm=8.0)
    P = Plan(p)
    assert P.z_mirror
    x = torch.from_numpy(PH.ellipsoids_3d(24, seed=5).reshape(-1)).cuda()
    b = P.adjoint(P.forward(x)).reshape(-1).contiguous()
    cg = NativeCGLS(P, mode)
    want = cg.solve(b, iters=4).cpu().numpy()
    u0 = (0.5 * x).contiguous()
    want0 = cg.solve(b, u0=u0, iters=3, zero_start=False).cpu().numpy()
    for pinned in (False, True):
        bh = torch.empty(b.numel(), dtype=torch.float32, pin_memory=pinned)
        uh = torch.full((b.numel(),), 7.0, dtype=torch.float32, pin_memory=pinned)
        bh.copy_(b.cpu())
        got = cg.solve_host(bh.numpy(), uh.numpy(), iters=4)
        assert np.array_equal(got, want), (mode, pinned)
        uh.copy_(u0.cpu())
        got0 = cg.solve_host(bh.numpy(), uh.numpy(), iters=3, zero_start=False)
        assert np.array_equal(got0, want0), (mode, pinned)
