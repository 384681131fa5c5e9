"""Generates tests/golden/*.npz from the reference's own CPU kernels.

Run where the reference checkout exists (it builds oracle/_ref from the
unmodified reference sources):  python tests/golden/make_golden.py
Every case is seeded; inputs are N(0,1) or an ellipse/ellipsoid phantom, the
geometry comes from framelab_gb300.geometry (the setPara.m mirror).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from framelab_gb300 import geometry as G  # noqa: E402
from framelab_gb300 import phantoms as PH  # noqa: E402
from tests.golden.fixtures import save_case  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def main():
    O.build(with_ref=True)
    if not O.have_ref():
        raise SystemExit("reference sources not available")
    rng = np.random.default_rng(20240601)

    # fan-beam, reference default scanner (SO = OD = 5, Ly = 6) on a 2x2 object
    p = G.fan_para(48, 48, 64, 24, L=(2, 2))
    x = rng.standard_normal(48 * 48).astype(np.float32)
    save_case(f"{OUT}/fan_siddon_rand.npz", "fan_siddon", p, x, O.ref_fan_siddon(x, p))
    save_case(f"{OUT}/fan_new_rand.npz", "fan_new", p, x, O.ref_fan_new(x, p))
    y = rng.standard_normal(64 * 24).astype(np.float32)
    save_case(f"{OUT}/fan_adj_rand.npz", "fan_adj", p, y, O.ref_fan_adj(y, p))

    # fan-beam, phantom, the 2-D benchmark geometry shrunk to 64^2 / 90 views
    pf = G.fan_para(64, 64, 128, 90, L=(1.0, 1.0), SO=500.0, OD=500.0, Ly=2 * np.sqrt(2))
    xf = PH.ellipses_2d(64, seed=7).reshape(-1)
    save_case(f"{OUT}/fan_siddon_phantom.npz", "fan_siddon", pf, xf, O.ref_fan_siddon(xf, pf))

    # cone-beam circle, reference default scanner, random volume
    pc = G.cone_para(24, 24, 24, 32, 28, 10, L=(2, 2, 2))
    xc = rng.standard_normal(24 ** 3).astype(np.float32)
    save_case(f"{OUT}/cone_siddon_rand.npz", "cone_siddon", pc, xc, O.ref_cone_siddon(xc, pc))
    yc, ycn = O.ref_cone_new(xc, pc)
    save_case(f"{OUT}/cone_new_rand.npz", "cone_new", pc, xc, yc, yNorm=ycn)
    yy = rng.standard_normal(32 * 28 * 10).astype(np.float32)
    save_case(f"{OUT}/cone_adj_rand.npz", "cone_adj", pc, yy, O.ref_cone_adj(yy, pc))

    # cone-beam helix, non-cubic voxels for the forward
    ph = G.cone_para(16, 16, 20, 24, 20, 0, L=(2, 2, 3), scan="helix", zmax=0.5, rps=1.0,
                     vtab=1.0, fps=12)
    xh = rng.standard_normal(16 * 16 * 20).astype(np.float32)
    save_case(f"{OUT}/cone_siddon_helix.npz", "cone_siddon", ph, xh, O.ref_cone_siddon(xh, ph))

    # cone-beam phantom in the 3-D benchmark geometry (mm units), shrunk
    pm = G.cone_para_mm(32, 12, 64, 48, det_pitch_mm=8.0, SO_mm=600.0, SD_mm=1200.0,
                        voxel_mm=8.0)
    xm = PH.ellipsoids_3d(32, seed=11).reshape(-1)
    save_case(f"{OUT}/cone_siddon_phantom.npz", "cone_siddon", pm, xm, O.ref_cone_siddon(xm, pm))
    ym = rng.standard_normal(64 * 48 * 12).astype(np.float32)
    save_case(f"{OUT}/cone_adj_mm.npz", "cone_adj", pm, ym, O.ref_cone_adj(ym, pm))
    # finite-size beam fan pair (version 2) on a phantom and an offset detector
    pb = G.fan_para(48, 48, 40, 24, L=(2, 2), SO=4.0, OD=3.0, Ly=6.0, y_os=0.21)
    xb = PH.ellipses_2d(48, seed=5).reshape(-1)
    save_case(f"{OUT}/fan_fb_phantom.npz", "fan_fb", pb, xb, O.ref_fan_fb(xb, pb))
    yb = rng.standard_normal(40 * 24).astype(np.float32)
    save_case(f"{OUT}/fan_fb_adj_rand.npz", "fan_fb_adj", pb, yb, O.ref_fan_fb_adj(yb, pb))
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))


if __name__ == "__main__":
    main()
