"""torch.autograd binding: gradient of 1/2|Ax - b|^2 vs central differences."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_gradient_matches_central_differences():
    import torch
    from framelab_gb300 import geometry as G, phantoms as PH
    from framelab_gb300.autograd import fd_gradcheck, project
    from framelab_gb300.projector import Plan
    p = G.cone_para_mm(48, 30, 72, 64, det_pitch_mm=5.0, SO_mm=600.0, SD_mm=1200.0, voxel_mm=5.0)
    P = Plan(p)
    x = torch.from_numpy(PH.ellipsoids_3d(48, seed=1)).cuda().reshape(P.vol_shape)
    b = project(x * 1.1 + 0.05, P).detach()
    err, idx = fd_gradcheck(P, x, b, n_vox=64, h=1e-3)
    assert err < 1e-3, err


def test_backward_is_the_adjoint():
    import torch
    from framelab_gb300 import geometry as G
    from framelab_gb300.autograd import project
    from framelab_gb300.projector import Plan
    p = G.fan_para(64, 64, 96, 40, L=(1.0, 1.0), SO=4.0, OD=4.0, Ly=3.0)
    P = Plan(p)
    x = torch.randn(P.vol_shape, device="cuda", requires_grad=True)
    w = torch.randn(P.sino_shape, device="cuda")
    (project(x, P) * w).sum().backward()
    assert torch.equal(x.grad, P.adjoint(w))
