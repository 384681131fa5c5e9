"""The MATLAB class mirror on the GPU: scanners reproduce the reference's CPU
projectors bit for bit through the class interface, and the generic CGLS /
split-Bregman loops (solveCGLS.m, solveSplitBregman.m) follow the FP64
restatement."""
import numpy as np
import pytest

import oracle as O
from oracle import numerics as N
from framelab_gb300 import phantoms as PH
from framelab_gb300.classes import DataTypes, Operators, Optimizers, Transforms

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().float().cpu().numpy().reshape(-1)


def test_cone_scanner_apply_and_adjoint_are_the_reference_kernels():
    cbct = Operators.ConeBeamScanner("circle", 40, 36, 12)
    x = PH.ellipsoids_3d(24, seed=1)
    u = DataTypes.ObjectData(3, x, [2, 2, 2])
    f = cbct.apply(u)
    assert tuple(f.dataArray.shape) == (12, 36, 40)
    y, yn = O.cone_gao_f32(x.reshape(-1), cbct.para)
    assert np.array_equal(_np(f.dataArray), y) and np.array_equal(_np(f.dataArrayNorm), yn)
    b = cbct.applyAdjoint(f, [24, 24, 24])
    assert b.N == (24, 24, 24)
    assert np.array_equal(_np(b.dataArray), O.cone_adj_f32(_np(f.dataArray), cbct.para))


def test_fan_scanner_versions_are_the_reference_kernels():
    x = PH.ellipses_2d(48, seed=2)
    u = DataTypes.ObjectData(2, x, [10, 10])
    for version, fwd, adj in ((0, O.fan_siddon_f32, O.fan_adj_f32),
                              (1, O.fan_gao_f32, O.fan_adj_f32),
                              (2, O.fan_fb_f32, O.fan_fb_adj_f32)):
        fbct = Operators.FanBeamScanner(96, 30, version=version)
        f = fbct.apply(u)
        assert tuple(f.dataArray.shape) == (30, 96)
        assert np.array_equal(_np(f.dataArray), fwd(x.reshape(-1), fbct.para)), version
        b = fbct.applyAdjoint(f)
        assert np.array_equal(_np(b.dataArray), adj(_np(f.dataArray), fbct.para)), version


def test_adjoint_refuses_data_of_another_geometry():
    u = DataTypes.ObjectData(2, PH.ellipses_2d(32, seed=3), [10, 10])
    a, c = Operators.FanBeamScanner(64, 16), Operators.FanBeamScanner(80, 16)
    fa = a.apply(u)
    c.apply(u)
    with pytest.raises(ValueError, match="do not agree"):
        c.applyAdjoint(fa)


def test_multihelix_data_shape():
    s = Operators.ConeBeamScanner("multiHelix", 24, 20, None, zmax=0.5, rps=1.0, vtab=1.0,
                                  fps=8, nHelix=2, phaseShift=(0.0, 1.0))
    f = s.apply(DataTypes.ObjectData(3, PH.ellipsoids_3d(16, seed=4), [2, 2, 2]))
    assert tuple(f.dataArray.shape) == (2, s.nv // 2, 20, 24)


def test_generic_cgls_follows_the_fp64_restatement():
    cbct = Operators.ConeBeamScanner("circle", 36, 32, 10, model="matched")
    n = 16
    x = PH.ellipsoids_3d(n, seed=5)
    u = DataTypes.ObjectData(3, x, [2, 2, 2])
    A = lambda o: cbct.apply(o)                                 # noqa: E731
    At = lambda d: cbct.applyAdjoint(d, [n, n, n])              # noqa: E731
    b = At(A(u))
    u0 = DataTypes.ObjectData(3, np.zeros((n, n, n), np.float32), [2, 2, 2])
    lam, iters = 0.5, 6
    cg = Optimizers.CGLS(A, At, b, u0, lam, iters, 1e-30)
    got = _np(cg.solveCGLS().dataArray)
    p = cbct.para
    bb = O.exact_adjoint(O.exact_forward(x.reshape(-1).astype(np.float64), p), p)
    want, _ = N.cgls(lambda v: O.exact_adjoint(O.exact_forward(v, p), p), bb,
                     np.zeros_like(bb), lam, iters)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-4
    assert len(cg.history) == iters


def test_generic_split_bregman_follows_the_fp64_restatement():
    cbct = Operators.ConeBeamScanner("circle", 36, 32, 10, model="matched")
    n = 16
    x = PH.ellipsoids_3d(n, seed=6)
    u = DataTypes.ObjectData(3, x, [2, 2, 2])
    A = lambda o: cbct.apply(o)                                 # noqa: E731
    At = lambda d: cbct.applyAdjoint(d, [n, n, n])              # noqa: E731
    sys = Transforms.FrameletSystem(3, "linear", 1)
    W = lambda o: o.frameletTransform(sys)                      # noqa: E731
    Wt = lambda a: DataTypes.ObjectData(3, a.adjointFrameletTransform(sys), [2, 2, 2])  # noqa: E731
    f = A(u)
    u0 = DataTypes.ObjectData(3, np.zeros((n, n, n), np.float32), [2, 2, 2])
    lam, mu = 0.01, 1.0
    sb = Optimizers.SplitBregman(A, At, W, Wt, lam, mu, f, u0, 3, 4, 1e-30)
    got = _np(sb.solveSplitBregman().dataArray)
    p = cbct.para
    Af = lambda v: O.exact_forward(v, p)                        # noqa: E731
    Atf = lambda y: O.exact_adjoint(y, p)                       # noqa: E731
    Wf = lambda v: N.frame_dec(v.reshape(n, n, n), 1, "linear")  # noqa: E731
    Wtf = lambda c: N.frame_rec(c, "linear").reshape(-1)        # noqa: E731
    fe = _np(f.dataArray).astype(np.float64)
    want = N.split_bregman(Af, Atf, Wf, Wtf, fe, np.zeros(n ** 3), lam, mu, 3, 4, 1e-30)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-3
