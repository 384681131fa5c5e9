"""Batched uneven fan-beam slices (fl_batch_*): every slice's forward/adjoint
equals its own plan's matched projector bit for bit, and the batched CGLS
follows the FP64 restatement of solveCGLS.m per slice."""
import numpy as np
import pytest

import oracle as O
from oracle import numerics as N
from framelab_gb300 import geometry as G
from framelab_gb300 import phantoms as PH

pytestmark = pytest.mark.gpu

# (nx, ny, nd, nv): uneven sizes, a rectangular image, odd detector widths
SLICES = [(16, 16, 33, 7), (24, 40, 61, 13), (40, 40, 81, 9), (32, 32, 64, 20), (20, 20, 41, 11)]


def _paras(slices=SLICES, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for nx, ny, nd, nv in slices:
        phi = np.sort(rng.uniform(0, 2 * np.pi, nv)).astype(np.float32)
        out.append(G.fan_para(nx, ny, nd, nv, L=(2.0 * nx / max(nx, ny), 2.0 * ny / max(nx, ny)),
                              SO=rng.uniform(3, 6), OD=rng.uniform(3, 6), Ly=rng.uniform(5, 8),
                              sd_phi=phi))
    return out


def _batch(paras):
    from framelab_gb300.batch import FanBatch
    return FanBatch(paras)


def test_batch_forward_adjoint_bit_identical_to_single_plans():
    import torch
    paras = _paras()
    B = _batch(paras)
    rng = np.random.default_rng(1)
    x = torch.from_numpy(rng.standard_normal(B.n_vox).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.standard_normal(B.n_rays).astype(np.float32)).cuda()
    yb, xb = B.forward(x), B.adjoint(y)
    torch.cuda.synchronize()
    for i, P in enumerate(B.plans):
        xi = B.images(x)[i].reshape(-1).contiguous()
        yi = B.sinograms(y)[i].reshape(-1).contiguous()
        assert torch.equal(B.sinograms(yb)[i].reshape(-1),
                           P.forward(xi, model="matched").reshape(-1)), i
        assert torch.equal(B.images(xb)[i].reshape(-1),
                           P.adjoint(yi, model="matched").reshape(-1)), i


# views evenly over a full turn: the slice plans take the quarter turn (square,
# nv a multiple of 4), the half turn (nv even) or neither (nv odd)
TURN_SLICES = [(32, 32, 64, 20), (24, 40, 61, 14), (40, 40, 81, 9), (48, 48, 96, 36),
               (20, 36, 41, 12)]


def _turn_paras(slices=TURN_SLICES, seed=0):
    rng = np.random.default_rng(seed)
    return [G.fan_para(nx, ny, nd, nv, L=(2.0 * nx / max(nx, ny), 2.0 * ny / max(nx, ny)),
                       SO=rng.uniform(3, 6), OD=rng.uniform(3, 6), Ly=rng.uniform(5, 8))
            for nx, ny, nd, nv in slices]


def test_batch_turn_slices_bit_identical_to_single_plans():
    import torch
    from framelab_gb300.batch import FanBatch
    paras = _turn_paras()
    B = FanBatch(paras)
    assert B.turns == [4, 2, 1, 4, 2] and B.launches_per_iteration == 8
    rng = np.random.default_rng(8)
    x = torch.from_numpy(rng.standard_normal(B.n_vox).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.standard_normal(B.n_rays).astype(np.float32)).cuda()
    yb, xb = B.forward(x), B.adjoint(y)
    torch.cuda.synchronize()
    for i, P in enumerate(B.plans):
        xi = B.images(x)[i].reshape(-1).contiguous()
        yi = B.sinograms(y)[i].reshape(-1).contiguous()
        assert torch.equal(B.sinograms(yb)[i].reshape(-1),
                           P.forward(xi, model="matched").reshape(-1)), i
        assert torch.equal(B.images(xb)[i].reshape(-1),
                           P.adjoint(yi, model="matched").reshape(-1)), i
    # without the turns every slice takes the general kernels, still bit for bit
    B1 = FanBatch(paras, turns=False)
    assert B1.turns == [1] * 5 and B1.launches_per_iteration == 6
    yb1 = B1.forward(x)
    for i, P in enumerate(B1.plans):
        xi = B1.images(x)[i].reshape(-1).contiguous()
        assert torch.equal(B1.sinograms(yb1)[i].reshape(-1),
                           P.forward(xi, model="matched").reshape(-1)), i
    # the two matrices differ only by the turned views' FP32 rounding, except
    # on an odd detector's central ray (it runs along a pixel boundary at view
    # angle 0, and the turn forms keep view 0's choice for its turned copies)
    for i, (_, _, nd, _) in enumerate(TURN_SLICES):
        a, b = B.sinograms(yb)[i], B1.sinograms(yb1)[i]
        if nd % 2:
            keep = torch.ones(nd, dtype=torch.bool, device=a.device)
            keep[nd // 2] = False
            a, b = a[:, keep], b[:, keep]
        assert float((a - b).norm() / b.norm()) < 1e-5, i


# views evenly over a full turn with symmetric detectors of even width: the
# reflection alone (odd nv, and a single view), with the quarter turns (nv a
# multiple of 8), with the half turn (with and without an end view), beside a
# quarter-turn slice (nv = 4 mod 8) and a general one (odd detector width)
REFL_SLICES = [(32, 32, 64, 37), (32, 32, 64, 40), (24, 40, 62, 14), (40, 24, 80, 12),
               (32, 32, 64, 44), (20, 20, 41, 11), (16, 16, 32, 1)]


def test_batch_reflection_slices_bit_identical_to_single_plans():
    """Slices whose plans use a reflection form run those forms' kernels in
    the batch (a third branch beside the turn and the general slices): each
    slice's forward and backprojection equal its plan's bit for bit, and the
    batched CGLS equals the single-slice graph solver's bits too."""
    import torch
    from framelab_gb300.batch import FanBatch
    from framelab_gb300.solvers import NativeCGLS
    rng = np.random.default_rng(3)
    paras = [G.fan_para(nx, ny, nd, nv, L=(1.0, ny / nx), SO=rng.uniform(3, 6),
                        OD=rng.uniform(3, 6), Ly=rng.uniform(5, 8))
             for nx, ny, nd, nv in REFL_SLICES]
    B = FanBatch(paras)
    assert B.turns == [2, 8, 4, 4, 4, 1, 2], B.turns
    assert B.reflect == [True, True, True, True, False, False, True]
    assert B.launches_per_iteration == 10
    x = torch.from_numpy(rng.standard_normal(B.n_vox).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.standard_normal(B.n_rays).astype(np.float32)).cuda()
    yb, xb = B.forward(x), B.adjoint(y)
    torch.cuda.synchronize()
    for i, P in enumerate(B.plans):
        xi = B.images(x)[i].reshape(-1).contiguous()
        yi = B.sinograms(y)[i].reshape(-1).contiguous()
        assert torch.equal(B.sinograms(yb)[i].reshape(-1),
                           P.forward(xi, model="matched").reshape(-1)), i
        assert torch.equal(B.images(xb)[i].reshape(-1),
                           P.adjoint(yi, model="matched").reshape(-1)), i
    b = B.adjoint(B.forward(x))
    ub = B.cgls(b, iters=4)
    for i, P in enumerate(B.plans):
        bi = B.images(b)[i].reshape(-1).contiguous()
        ui = NativeCGLS(P, "graph").solve(bi, iters=4)
        assert float((B.images(ub)[i].reshape(-1) - ui).norm() / ui.norm()) < 1e-5, i
    # the batch tuner covers the reflection slices' parts too
    parts = B.autotune()
    assert parts in (1, 4, 16)
    for P, t in zip(B.plans, B.turns):
        if t > 1:
            P.set_tuning("fan_parts", parts)
    yb = B.forward(x)
    for i, P in enumerate(B.plans):
        xi = B.images(x)[i].reshape(-1).contiguous()
        assert torch.equal(B.sinograms(yb)[i].reshape(-1),
                           P.forward(xi, model="matched").reshape(-1)), i


def test_batch_autotune_and_parts_keep_batch_equal_to_plans():
    """A batch takes its turn slices' parts per walked ray from their plans
    (here set to 4), and its own tuner sets one count for all of them; either
    way each slice's forward equals its plan's with that count, bit for bit,
    and the backprojection is unchanged."""
    import torch
    from framelab_gb300.batch import FanBatch
    paras = _turn_paras()
    B = FanBatch(paras, fan_parts=4)
    rng = np.random.default_rng(9)
    x = torch.from_numpy(rng.standard_normal(B.n_vox).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.standard_normal(B.n_rays).astype(np.float32)).cuda()

    def check():
        yb, xb = B.forward(x), B.adjoint(y)
        torch.cuda.synchronize()
        for i, P in enumerate(B.plans):
            xi = B.images(x)[i].reshape(-1).contiguous()
            yi = B.sinograms(y)[i].reshape(-1).contiguous()
            assert torch.equal(B.sinograms(yb)[i].reshape(-1),
                               P.forward(xi, model="matched").reshape(-1)), i
            assert torch.equal(B.images(xb)[i].reshape(-1),
                               P.adjoint(yi, model="matched").reshape(-1)), i

    assert [P.tuning("fan_parts") for P, t in zip(B.plans, B.turns) if t > 1] == [4] * 4
    check()
    b = torch.from_numpy(rng.standard_normal(B.n_vox).astype(np.float32)).cuda()
    B.cgls(b, iters=3)                    # captures its graph with 4 parts
    parts = B.autotune()
    assert parts in (1, 4, 16)
    for P, t in zip(B.plans, B.turns):
        if t > 1:
            P.set_tuning("fan_parts", parts)
    check()
    # the CUDA-graph CGLS is recaptured with the new work list
    u1 = B.cgls(b, iters=3)
    B2 = FanBatch(paras, fan_parts=parts)
    u2 = B2.cgls(b, iters=3)
    assert torch.equal(u1, u2)
    assert FanBatch(paras, turns=False).autotune() == 0


def test_batch_tiny_slices_of_every_kind_bit_identical():
    """Degenerate slices in one batch: one view (general), a one-pixel-wide
    image (general: the turns need even nx and ny), a single detector column
    over a 2 x 2 image (half turn), a 2 x 2 image (quarter turn), beside a
    normal slice, and 2 x 2 images with the reflection alone (3 views) and
    with the quarter turns (8 views: the one primary pixel is on the
    diagonal)."""
    import torch
    from framelab_gb300.batch import FanBatch
    paras = [G.fan_para(2, 2, 3, 1, L=(1.0, 1.0), SO=3.0, OD=3.0, Ly=3.0, y_os=0.013),
             G.fan_para(1, 2, 1, 2, L=(1.0, 2.0), SO=3.0, OD=3.0, Ly=3.0, y_os=0.013),
             G.fan_para(2, 2, 1, 2, L=(1.0, 1.0), SO=3.0, OD=3.0, Ly=3.0, y_os=0.013),
             G.fan_para(2, 2, 2, 4, L=(1.0, 1.0), SO=3.0, OD=3.0, Ly=3.0),
             G.fan_para(24, 24, 48, 12, L=(1.0, 1.0), SO=3.0, OD=3.0, Ly=3.0),
             G.fan_para(2, 2, 2, 3, L=(1.0, 1.0), SO=3.0, OD=3.0, Ly=3.0),
             G.fan_para(2, 2, 2, 8, L=(1.0, 1.0), SO=3.0, OD=3.0, Ly=3.0)]
    B = FanBatch(paras)
    assert B.turns == [1, 1, 2, 4, 4, 2, 8]
    rng = np.random.default_rng(14)
    x = torch.from_numpy(rng.standard_normal(B.n_vox).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.standard_normal(B.n_rays).astype(np.float32)).cuda()
    yb, xb = B.forward(x), B.adjoint(y)
    torch.cuda.synchronize()
    for i, P in enumerate(B.plans):
        xi = B.images(x)[i].reshape(-1).contiguous()
        yi = B.sinograms(y)[i].reshape(-1).contiguous()
        assert torch.equal(B.sinograms(yb)[i].reshape(-1),
                           P.forward(xi, model="matched").reshape(-1)), i
        assert torch.equal(B.images(xb)[i].reshape(-1),
                           P.adjoint(yi, model="matched").reshape(-1)), i
    u = B.cgls(B.adjoint(B.forward(torch.abs(x))), lam=0.1, iters=3)
    assert bool(torch.isfinite(u).all())


def test_batch_turn_slices_cgls_agree_with_single_slice_solver():
    import torch
    from framelab_gb300.batch import FanBatch
    from framelab_gb300.solvers import NativeCGLS
    B = FanBatch(_turn_paras(seed=9))
    rng = np.random.default_rng(10)
    rhs = torch.from_numpy(rng.uniform(0, 1, B.n_vox).astype(np.float32)).cuda()
    u = B.cgls(rhs, lam=0.5, iters=6)
    assert list(B.iters_done) == [6] * len(B)
    for i, P in enumerate(B.plans):
        ri = B.images(rhs)[i].reshape(-1).contiguous()
        ui = NativeCGLS(P, "graph").solve(ri, lam=0.5, iters=6)
        got = B.images(u)[i].reshape(-1)
        rel = float((got - ui).norm() / ui.norm())
        assert rel < 1e-5, (i, rel)
    # a warm start runs the turn slices' forward and adjoint outside the graph
    u2 = B.cgls(rhs, lam=0.5, iters=2, u0=u)
    assert bool(torch.isfinite(u2).all())


def test_batch_cgls_matches_fp64_oracle_per_slice():
    import torch
    paras = _paras(SLICES[:4], seed=2)
    B = _batch(paras)
    lam, iters = 0.1, 8
    rhs, want = [], []
    for i, p in enumerate(paras):
        nx, ny = int(p["nx"]), int(p["ny"])
        x = PH.ellipses_2d(nx, seed=i) if nx == ny else np.random.default_rng(i).uniform(0, 1, (ny, nx))
        b = O.exact_adjoint(O.exact_forward(x.reshape(-1).astype(np.float64), p), p)
        rhs.append(b)
        normal = lambda v, p=p: O.exact_adjoint(O.exact_forward(v, p), p)  # noqa: E731
        want.append(N.cgls(normal, b, np.zeros_like(b), lam, iters)[0])
    u = B.cgls(torch.from_numpy(np.concatenate(rhs).astype(np.float32)).cuda(), lam=lam,
               iters=iters).cpu().numpy()
    assert list(B.iters_done) == [iters] * len(paras)
    for i, w in enumerate(want):
        ui = u[B.vox_offsets[i]:B.vox_offsets[i + 1]]
        rel = np.linalg.norm(ui - w) / np.linalg.norm(w)
        # FP32 model and arithmetic against the FP64 exact pair: 8 CG steps on
        # an underdetermined fan system amplify the ~1e-6 entry differences
        assert rel < 1e-3, (i, rel)
        g = B.history[i]
        assert np.all(np.isfinite(g)) and g[-1] < g[0]


def test_batch_cgls_agrees_with_single_slice_solver():
    import torch
    from framelab_gb300.solvers import NativeCGLS
    paras = _paras(seed=3)
    B = _batch(paras)
    rng = np.random.default_rng(4)
    rhs = torch.from_numpy(rng.uniform(0, 1, B.n_vox).astype(np.float32)).cuda()
    u = B.cgls(rhs, lam=0.5, iters=6)
    for i, P in enumerate(B.plans):
        ri = B.images(rhs)[i].reshape(-1).contiguous()
        ui = NativeCGLS(P, "graph").solve(ri, lam=0.5, iters=6)
        got = B.images(u)[i].reshape(-1)
        rel = float((got - ui).norm() / ui.norm())
        assert rel < 1e-5, (i, rel)


def test_batch_slices_stop_independently_and_warm_start():
    import torch
    paras = _paras(seed=5)
    B = _batch(paras)
    rng = np.random.default_rng(6)
    rhs = torch.from_numpy(rng.uniform(0, 1, B.n_vox).astype(np.float32)).cuda()
    B.images(rhs)[2].zero_()            # a slice with nothing to solve stops at once
    u = B.cgls(rhs, lam=1.0, iters=5)
    assert B.iters_done[2] == 0 and all(B.iters_done[i] == 5 for i in (0, 1, 3, 4))
    assert float(B.images(u)[2].abs().max()) == 0.0
    u3 = B.cgls(rhs, lam=1.0, iters=3)
    u6 = B.cgls(rhs, lam=1.0, iters=3, u0=u3)
    u6_direct = B.cgls(rhs, lam=1.0, iters=6)
    rel = float((u6 - u6_direct).norm() / u6_direct.norm())
    assert rel < 0.2                    # a warm restart lands near the 6-iteration solution
