"""Runs every form of the matched projector pair, the batched fan kernels
and the fused CGLS through the bounds-checked library (started with
FRAMELAB_GB300_VARIANT=checked) and prints the number of out-of-range gathers
the kernels counted. Used by tests/test_gpu_bounds.py."""
import ctypes as C
import os
import sys

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from framelab_gb300 import _lib  # noqa: E402
from framelab_gb300 import geometry as G  # noqa: E402
from framelab_gb300.batch import FanBatch  # noqa: E402
from framelab_gb300.classes import DataTypes, Operators  # noqa: E402
from framelab_gb300.projector import Plan  # noqa: E402
from framelab_gb300.solvers import NativeCGLS  # noqa: E402


def run_plan(p, rng):
    P = Plan(p)
    x = torch.from_numpy(rng.standard_normal(P.n_vox).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.standard_normal(P.n_rays).astype(np.float32)).cuda()
    for dt in (torch.float32, torch.float16):
        P.forward(x.to(dt))
        P.adjoint(y.to(dt))
    if P.cone:                         # every symmetry level the plan allows
        for f, q, r, z in ((False, True, True, True), (True, False, True, True),
                           (False, False, True, True), (False, False, False, True),
                           (False, False, False, False)):
            P.reflect, P.quarter_turn, P.rot_mirror, P.z_mirror = f, q, r, z
            P.forward(x)
            P.adjoint(y)
            P.adjoint(y.half())
        P.z_mirror, P.rot_mirror, P.quarter_turn, P.reflect = True, True, True, True
    else:                              # fan: every form the plan allows
        for f, q, r in ((False, True, True), (True, False, True), (False, False, True),
                        (True, False, False), (False, False, False)):
            P.reflect, P.quarter_turn, P.rot_mirror = f, q, r
            P.forward(x)
            P.adjoint(y)
        P.rot_mirror, P.quarter_turn, P.reflect = True, True, True
    for mode in ("graph", "mixed"):
        NativeCGLS(P, mode).solve(torch.abs(x), lam=0.1, iters=3, refresh=2)


def main():
    L = _lib.load()
    v = C.c_int64()
    st = L.fl_debug_bounds(C.byref(v), 1)
    assert st == _lib.FL_OK, "not a bounds-checked build"
    rng = np.random.default_rng(0)
    cases = [
        G.cone_para_mm(32, 16, 48, 40, det_pitch_mm=8.0, SO_mm=600.0, SD_mm=1200.0,
                       voxel_mm=8.0),                                  # circle: reflection
        G.cone_para_mm(24, 8, 32, 28, det_pitch_mm=8.0, SO_mm=600.0, SD_mm=1200.0,
                       voxel_mm=8.0),                                  # reflection, nv = 8
        G.cone_para_mm(32, 12, 48, 40, det_pitch_mm=8.0, SO_mm=600.0, SD_mm=1200.0,
                       voxel_mm=8.0),                                  # quarter turns
        G.cone_para(32, 24, 16, 40, 36, 18, L=(2.0, 1.5, 1.0)),        # half turn, reflection
        G.cone_para_mm(28, 18, 44, 36, det_pitch_mm=8.0, SO_mm=600.0, SD_mm=1200.0,
                       voxel_mm=8.0),                                  # circle: half turn
        G.cone_para(16, 16, 16, 36, 32, 10, L=(2, 2, 2)),              # short SO, steep rows
        G.cone_para(20, 18, 14, 30, 26, 0, L=(2, 2, 2), scan="helix", zmax=0.5, rps=1.0,
                    vtab=1.0, fps=8),                                  # helix: general kernels
        G.cone_para_mm(24, 12, 40, 33, det_pitch_mm=6.0, SO_mm=500.0, SD_mm=1000.0,
                       voxel_mm=6.0, nz=17),                           # odd nz and nb
        G.fan_para(64, 64, 128, 30, L=(1, 1)),                         # fan, 1 x 1 blocks
        G.fan_para(512, 512, 1024, 60, L=(1, 1)),                      # fan, 2 x 2 blocks
        G.fan_para(48, 36, 97, 42, L=(1, 0.75), SO=3.0, OD=3.0, Ly=3.0),  # fan, rectangular
        G.fan_para(640, 480, 64, 6, L=(1, 0.75), SO=3.0, OD=3.0, Ly=3.0),  # fan, 2 x 2 turn blocks
        G.fan_para(64, 64, 128, 31, L=(1, 1)),                         # fan, reflection alone
        G.fan_para(64, 64, 128, 32, L=(1, 1)),                         # fan, quarter turns + refl.
        G.fan_para(48, 36, 96, 40, L=(1, 0.75), SO=3.0, OD=3.0, Ly=3.0),  # half turn + refl., end view
        G.fan_para(512, 512, 1024, 61, L=(1, 1)),                      # reflection alone, large
    ]
    for p in cases:
        run_plan(p, rng)
    sl = [(16, 16, 33, 7), (24, 40, 61, 13), (40, 40, 81, 9)]
    B = FanBatch([G.fan_para(nx, ny, nd, nv, L=(2.0 * nx / max(nx, ny), 2.0 * ny / max(nx, ny)))
                  for nx, ny, nd, nv in sl])
    xb = torch.rand(B.n_vox, device="cuda")
    B.adjoint(B.forward(xb))
    B.cgls(B.adjoint(B.forward(xb)), iters=3)
    # a batch with half- and quarter-turn slices (views evenly over a full turn)
    sl = [(32, 32, 64, 20), (24, 40, 61, 14), (40, 40, 81, 9), (20, 36, 41, 12)]
    B = FanBatch([G.fan_para(nx, ny, nd, nv, L=(2.0 * nx / max(nx, ny), 2.0 * ny / max(nx, ny)))
                  for nx, ny, nd, nv in sl])
    assert B.turns == [4, 2, 1, 2], B.turns
    xb = torch.rand(B.n_vox, device="cuda")
    B.adjoint(B.forward(xb))
    B.cgls(B.adjoint(B.forward(xb)), iters=3)
    # a batch with reflection slices of every form beside turn and general ones
    sl = [(32, 32, 64, 37), (32, 32, 64, 40), (24, 40, 62, 14), (40, 24, 80, 12),
          (32, 32, 64, 44), (20, 20, 41, 11), (16, 16, 32, 1)]
    B = FanBatch([G.fan_para(nx, ny, nd, nv, L=(1.0, ny / nx), SO=3.0, OD=3.0, Ly=3.0)
                  for nx, ny, nd, nv in sl])
    assert B.turns == [2, 8, 4, 4, 4, 1, 2], B.turns
    xb = torch.rand(B.n_vox, device="cuda")
    B.adjoint(B.forward(xb))
    B.cgls(B.adjoint(B.forward(xb)), iters=3)
    for parts in (1, 4, 16):
        Bp = FanBatch([G.fan_para(nx, ny, nd, nv, L=(1.0, ny / nx), SO=3.0, OD=3.0, Ly=3.0)
                       for nx, ny, nd, nv in sl], fan_parts=parts)
        Bp.adjoint(Bp.forward(xb))
    B.autotune()
    B.cgls(B.adjoint(B.forward(xb)), iters=3)
    # the class mirror's default scanner geometry
    cb = Operators.ConeBeamScanner("circle", 36, 32, 10, model="matched")
    u = DataTypes.ObjectData(3, np.ones((16, 16, 16), np.float32), [2, 2, 2])
    cb.applyAdjoint(cb.apply(u), [16, 16, 16])
    torch.cuda.synchronize()
    _lib.check(L.fl_debug_bounds(C.byref(v), 0))
    print("violations", v.value)


if __name__ == "__main__":
    main()
