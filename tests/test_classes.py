"""Argument checking of the MATLAB class mirror (no GPU work): the
constructors raise the reference classes' errors."""
import pytest

from framelab_gb300.classes import DataTypes, Operators, Optimizers, Transforms


def test_cone_scanner_constructor_errors():
    with pytest.raises(ValueError, match="You must specify type, na, nb and nv"):
        Operators.ConeBeamScanner("circle", 64, 64)
    with pytest.raises(ValueError, match="circle, helix and multiHelix are only valid types"):
        Operators.ConeBeamScanner("spiral", 64, 64, 32)
    with pytest.raises(ValueError, match="zmax, rps, vtab, fps are for helical scan only"):
        Operators.ConeBeamScanner("circle", 64, 64, 32, zmax=1.0)
    with pytest.raises(ValueError, match="helix and multiHelix require more inputs"):
        Operators.ConeBeamScanner("helix", 64, 64, 32)


def test_helical_view_counts_follow_the_class():
    # ConeBeamScanner.m:53-58: floor(fps*zmax/vtab)+1 per helix
    s = Operators.ConeBeamScanner("helix", 32, 32, None, zmax=1.0, rps=1.0, vtab=1.0, fps=16)
    assert s.nv == 17
    m = Operators.ConeBeamScanner("multiHelix", 32, 32, None, zmax=1.0, rps=1.0, vtab=1.0,
                                  fps=16, nHelix=2, phaseShift=(0.0, 3.14159))
    assert m.nv == 34


def test_solver_and_transform_constructor_errors():
    with pytest.raises(ValueError, match="CGLS requires A, At, b, u0 and lam"):
        Optimizers.CGLS(abs, abs)
    with pytest.raises(ValueError, match="SplitBregman requires A,At,W,Wt,lam,f,and u0"):
        Optimizers.SplitBregman(abs, abs, abs, abs)
    with pytest.raises(ValueError):
        Transforms.FrameletSystem(3, "spline", 1)
    assert DataTypes.ObjectData is not None
