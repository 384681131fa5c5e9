"""Framelet transform, shrink/Bregman step and split Bregman on the GPU against
the FP64 restatement (oracle/numerics.py)."""
import zlib

import numpy as np
import pytest

from oracle import numerics as N

pytestmark = pytest.mark.gpu


def _coef_flat(coefs, levels, dim):
    """Oracle coefficient list -> the library's flat layout."""
    out = []
    for l, lev in enumerate(coefs):
        last = l == levels - 1
        keys = sorted(lev.keys())  # (i, j, k) lexicographic = 9i + 3j + k
        for key in keys:
            if key == (0,) * dim and not last:
                continue
            out.append(lev[key].reshape(-1))
    return np.concatenate(out)


def _oracle_dec(u, levels, kind="linear"):
    return N.frame_dec(u, levels, kind)


@pytest.mark.parametrize("levels", [1, 2])
@pytest.mark.parametrize("kind", ["linear", "haar", "cubic"])
def test_framelet_3d_matches_oracle_and_reconstructs(levels, kind):
    import torch
    from framelab_gb300.transforms import FrameletSystem
    rng = np.random.default_rng(levels)
    u = rng.standard_normal((12, 20, 16)).astype(np.float32)
    fs = FrameletSystem(u.shape, kind, levels)
    ud = torch.from_numpy(u).cuda()
    c = fs.forward(ud)
    want = _coef_flat(N.frame_dec(u.astype(np.float64), levels, kind), levels, 3)
    got = c.cpu().numpy()
    assert got.size == want.size
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()
    rec = fs.adjoint(c).cpu().numpy()
    assert np.linalg.norm(rec - u) / np.linalg.norm(u) < 1e-6      # W^T W = I (testFramelet.m:31)


def test_framelet_2d_matches_oracle():
    import torch
    from framelab_gb300.transforms import FrameletSystem
    rng = np.random.default_rng(3)
    u = rng.standard_normal((24, 18)).astype(np.float32)
    fs = FrameletSystem(u.shape, "linear", 2)
    c = fs.forward(torch.from_numpy(u).cuda()).cpu().numpy()
    # 2-D oracle: band (i, j) = D_i along x, D_j along y (FraDecMultiLevel2D.m)
    D, _ = N.filters("linear")
    coefs, cur = [], u.astype(np.float64)
    for lev in (1, 2):
        d = {}
        for i in range(3):
            ti = N.corr_circ(cur, D[i], -1, lev)
            for j in range(3):
                d[(i, j)] = N.corr_circ(ti, D[j], -2, lev)
        coefs.append(d)
        cur = d[(0, 0)]
    want = _coef_flat(coefs, 2, 2)
    assert np.abs(c - want).max() <= 1e-5 * np.abs(want).max()
    rec = fs.adjoint(torch.from_numpy(c).cuda()).cpu().numpy()
    assert np.linalg.norm(rec - u) / np.linalg.norm(u) < 1e-6


def test_bregman_step_matches_oracle():
    import torch
    from framelab_gb300.transforms import FrameletSystem
    rng = np.random.default_rng(9)
    shape, levels, mu, tau = (10, 12, 14), 2, 0.7, 0.05
    u = rng.standard_normal(shape)
    v0 = N.frame_dec(rng.standard_normal(shape), levels)
    Atf = rng.standard_normal(shape)
    # oracle: alpha = shrink(v + Wu); v' = v + Wu - alpha; b = Atf + mu W^T(alpha - v')
    Wu = N.frame_dec(u, levels)
    alpha = N.shrink(N.coef_add(v0, Wu), tau)
    v1 = N.coef_add(v0, N.coef_add(Wu, alpha, 1.0, -1.0))
    b = Atf + mu * N.frame_rec(N.coef_add(alpha, v1, 1.0, -1.0))
    fs = FrameletSystem(shape, "linear", levels)
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()  # noqa: E731
    v = cu(_coef_flat(v0, levels, 3))
    t = torch.empty_like(v)
    bo = torch.empty(shape, device="cuda")
    fs.bregman(cu(u), v, t, cu(Atf), mu, tau, bo)
    assert np.abs(v.cpu().numpy() - _coef_flat(v1, levels, 3)).max() < 1e-5
    assert np.linalg.norm(bo.cpu().numpy() - b) / np.linalg.norm(b) < 1e-5


def test_split_bregman_matches_oracle():
    import torch
    import oracle as O
    from framelab_gb300 import geometry as G, phantoms as PH
    from framelab_gb300.projector import Plan
    from framelab_gb300.transforms import split_bregman
    n = 16
    p = G.cone_para_mm(n, 12, 24, 20, det_pitch_mm=16.0, SO_mm=600.0, SD_mm=1200.0, voxel_mm=16.0)
    x = PH.ellipsoids_3d(n, seed=3).reshape(-1).astype(np.float64)
    f = O.exact_forward(x, p, threads=8)
    A = lambda v: O.exact_forward(v.reshape(-1), p, threads=8)  # noqa: E731
    At = lambda y: O.exact_adjoint(y, p, threads=8).reshape(n, n, n)  # noqa: E731
    W = lambda v: N.frame_dec(v.reshape(n, n, n), 2)  # noqa: E731
    Wt = lambda c: N.frame_rec(c)  # noqa: E731
    lam, mu, outer, cgi = 0.05, 1.0, 3, 4

    def A_flat(v):
        return A(v)

    def At_flat(y):
        return At(y).reshape(-1)

    u64 = N.split_bregman(A_flat, At_flat, lambda v: W(v), lambda c: Wt(c).reshape(-1), f,
                          np.zeros(n ** 3), lam, mu, outer, cgi)
    P = Plan(p)
    fd = torch.from_numpy(f.astype(np.float32)).cuda()
    for mode in ("plain", "mixed"):
        u, hist = split_bregman(P, fd, torch.zeros(n ** 3, device="cuda"), lam, mu, outer, cgi,
                                levels=2, mode=mode)
        u = u.cpu().numpy()
        rel = np.linalg.norm(u - u64) / np.linalg.norm(u64)
        assert rel < (1e-4 if mode == "plain" else 2e-3), (mode, rel)
        assert np.all(np.isfinite(hist)) and hist.size == outer


# z-streaming kernels (3-D levels of the three-tap banks, dilation up to 8)
# against the separable pass per axis: the same fmaf chains, so identical
# bits. Shapes cover ragged column tiles, fewer slices than a residue class
# needs and fewer columns than a warp; level 5 (dilation 16) and the cubic
# bank take the separable passes in both forms.
FUSED_SHAPES = [(12, 20, 16), (9, 37, 70), (3, 5, 40), (17, 8, 33)]


@pytest.mark.parametrize("shape", FUSED_SHAPES)
@pytest.mark.parametrize("kind", ["linear", "haar", "cubic"])
@pytest.mark.parametrize("levels", [1, 2, 4, 5])
def test_fused_levels_bit_identical_to_separable(shape, kind, levels):
    import torch
    from framelab_gb300.transforms import FrameletSystem
    rng = np.random.default_rng(zlib.crc32(repr((shape, kind, levels)).encode()))
    u = torch.from_numpy(rng.standard_normal(shape).astype(np.float32)).cuda()
    Atf = torch.from_numpy(rng.standard_normal(shape).astype(np.float32)).cuda()
    fs = FrameletSystem(shape, kind, levels)
    out = {}
    for fused in (True, False):
        fs.fused = fused
        c = fs.forward(u)
        r = fs.adjoint(c)
        v = c * 0.5
        t = torch.empty_like(v)
        b = torch.empty(shape, device="cuda")
        fs.bregman(u, v, t, Atf, 0.8, 0.05, b)
        torch.cuda.synchronize()
        out[fused] = (c, r, v, t, b)
    for a, bb, what in zip(out[True], out[False], ("W u", "W^T c", "v", "t", "b")):
        assert torch.equal(a, bb), what


def test_fused_reconstructs_large_volume():
    import torch
    from framelab_gb300.transforms import FrameletSystem
    g = torch.Generator(device="cuda").manual_seed(5)
    u = torch.randn((96, 160, 128), device="cuda", generator=g)
    fs = FrameletSystem(tuple(u.shape), "linear", 2)
    c = fs.forward(u)
    rec = fs.adjoint(c)
    assert float((rec - u).norm() / u.norm()) < 1e-6               # W^T W = I
    fs.fused = False
    assert torch.equal(fs.forward(u), c)


def test_persistent_split_bregman_matches_one_shot():
    import torch
    from framelab_gb300 import geometry as G, phantoms as PH
    from framelab_gb300.projector import Plan
    from framelab_gb300.transforms import SplitBregmanSolver, split_bregman
    n = 24
    p = G.cone_para_mm(n, 16, 36, 30, det_pitch_mm=12.0, SO_mm=600.0, SD_mm=1200.0,
                       voxel_mm=12.0)
    P = Plan(p)
    x = torch.from_numpy(PH.ellipsoids_3d(n, seed=4).reshape(-1)).cuda()
    f = P.forward(x)
    u0 = torch.zeros(P.n_vox, device="cuda")
    kw = dict(lam=0.02, mu=1.0, outer=3, cg_iters=3)
    one, hist = split_bregman(P, f, u0, levels=2, mode="graph", **kw)
    S = SplitBregmanSolver(P, levels=2, kind="linear", mode="graph")
    a = S.solve(f, u0, **kw)
    b = S.solve(f, u0, **kw)                   # the workspace is reused
    torch.cuda.synchronize()
    assert torch.equal(a, one) and torch.equal(b, one)
    assert np.array_equal(S.history, hist)
