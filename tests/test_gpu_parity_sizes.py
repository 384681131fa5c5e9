"""Parity of the matched projector pair at the configurations' own sizes.

C1: 256^2 fan, 360 views x 512 bins, SO = OD = 500 mm, in full, on a 256 mm
field (1 mm pixels) and on the unit field (SO = 128,000 pixels, nearly
parallel rays); C2: 256^3 cone, 360 views x 512 x 384 at 1 mm; C5: 512^3
cone, 720 views x 1024 x 768 at 0.5 mm. The cone volumes are checked on
seeded random subsets of rays (forward) and voxels (backprojection), the
oracle evaluating each sampled entry exactly as its full function would.

For every operator three relative L2 errors are measured (oracle/parity.py):
the GPU result against the FP64 exact model, the reference's own FP32 CPU
kernel against the FP64 model, and the GPU result against the reference.
Each configuration runs twice. With the half and quarter turns (and the
reflection) off (the general and z-mirror kernels) the matched pair must be within 1e-5 of the
FP64 model everywhere, for the backprojection of the phantom's sinogram and
of N(0, 1) noise alike. With the turns on (the default) it projects the scan
whose turned views are exact turns of the walked ones (oracle/parity.py,
``snapped``): there it must be within 1e-5 of that scan's FP64 model
everywhere, and within 1e-5 of the nominal model for the forward and the
phantom's sinogram; the backprojection of noise then shows the angle snap
(up to 2.4e-7 rad at radius r), bounded here by 3e-4.
Against the reference the pair must be within 1e-5 or, where the reference
is itself further than that from the FP64 model (its FP32 Siddon at SO =
128,000 pixels; its chord backprojector, Atx_cone_mf_cpu_new.cpp:23-85 with
find_l_3d.cpp:94-182, drops the chords of rays that leave a voxel within a
rounding of an edge), within the reference's own error plus 1e-5 -- plus
the snap's own difference for the turn plans.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _ops(P):
    import torch

    def fwd(x):
        return P.forward(torch.from_numpy(np.ascontiguousarray(x)).cuda()).cpu().numpy()

    def adj(y):
        return P.adjoint(torch.from_numpy(np.ascontiguousarray(y)).cuda()).cpu().numpy()
    return fwd, adj


def _turns(P):
    return P.views_per_walk


def _check(res, turns):
    for op, r in res.items():
        if turns == 1:
            assert r["matched_vs_fp64"] < TOL, (op, r)
            assert r["matched_vs_reference"] < max(TOL, r["reference_vs_fp64"] + TOL), (op, r)
        else:
            assert r["matched_vs_fp64_snapped"] < TOL, (op, r)
            snap = 3e-4 if op == "adjoint_random_sino" else TOL
            assert r["matched_vs_fp64"] < snap, (op, r)
            assert r["matched_vs_reference"] < max(snap, r["reference_vs_fp64"] + snap), (op, r)


def _plans(p, fan_reflect=False):
    """The default plan, the plan without its turns (and reflection) and, for a
    fan scan with fan_reflect, the plan with the reflection taken."""
    from framelab_gb300.projector import Plan
    for form in ("default", "general") + (("reflect",) if fan_reflect else ()):
        P = Plan(p)
        if form == "general":
            P.quarter_turn = False
            P.rot_mirror = False
            P.reflect = False
        elif form == "reflect":
            P.reflect = True
        yield P


@pytest.mark.parametrize("field_mm", [256.0, 1.0])
def test_fan256_full(field_mm):
    import oracle.parity as PAR
    from framelab_gb300 import geometry as G, phantoms as PH
    L = field_mm
    p = G.fan_para(256, 256, 512, 360, L=(L, L), SO=500.0, OD=500.0,
                   Ly=2.0 * math.sqrt(2.0) * L)
    x = PH.ellipses_2d(256, seed=1)
    forms = []
    for P in _plans(p, fan_reflect=True):
        t = _turns(P)
        forms.append(t)
        _check(PAR.fan_parity(p, x, *_ops(P), turns=P.rotations, reflect=P.reflect), t)
    assert forms == [4, 1, 8]


@pytest.mark.parametrize("n", [256, 512])
def test_cone_config_sizes_on_subsets(n):
    import torch
    import oracle.parity as PAR
    from framelab_gb300 import geometry as G, phantoms as PH
    if n == 256:
        p = G.cone_para_mm(256, 360, 512, 384, det_pitch_mm=1.0, SO_mm=600.0, SD_mm=1200.0,
                           voxel_mm=1.0)
    else:
        p = G.cone_para_mm(512, 720, 1024, 768, det_pitch_mm=0.5, SO_mm=600.0, SD_mm=1200.0,
                           voxel_mm=0.5)
    x = PH.ellipsoids_3d(n, seed=1)
    forms = []
    for P in _plans(p):
        t = _turns(P)
        forms.append(t)
        res = PAR.cone_parity(p, x, *_ops(P), n_rays=20000, n_vox=4000 if n == 256 else 2000,
                              turns=P.rotations, reflect=P.reflect)
        del P
        torch.cuda.empty_cache()
        _check(res, t)
    assert forms == [8, 1]
