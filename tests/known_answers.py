"""Shared set-up of the reference's analytic known answers (testBall.m)."""
import numpy as np

from framelab_gb300 import geometry as G
from framelab_gb300 import phantoms as PH


def fan_disc(N=400, nd=200):
    """testBall.m:2-22: unit disc on a 2x2 object, default fan scanner, one view."""
    p = G.fan_para(N, N, nd, 1, L=(2, 2))
    x = PH.unit_ball(N, 2).reshape(-1)
    a = p["y_det"].astype(np.float64) * float(p["scale"])
    return p, x, PH.fan_disc_chord(a, 5.0, 5.0)


def fan_disc_beam(N=400, nd=200, sub=64):
    """The unit disc through the finite-size beam model: each bin integrates
    the chord over its wedge, whose width at the chord midpoint (distance
    SO*cos(g) from the source) is SO*cos(g)^3/SD per unit of detector, so the
    answer is the bin average of chord * SO*cos(g)^3/SD times the bin width
    in pixels (midpoint rule over ``sub`` sub-rays)."""
    p, x, _ = fan_disc(N, nd)
    sc, SO, SD = float(p["scale"]), 5.0, 10.0
    dy = float(p["dy_det"])
    a = p["y_det"].astype(np.float64) * sc
    u = a[:, None] + ((np.arange(sub) + 0.5) / sub - 0.5)[None, :] * dy * sc
    ch = PH.fan_disc_chord(u.reshape(-1), SO, SD - SO).reshape(u.shape)
    g = np.arctan2(u, SD)
    return p, x, (ch * SO * np.cos(g) ** 3 / SD).mean(1) * dy


def cone_ball(N=64, nd=64, scan="circle"):
    """testBall.m:23-78: unit ball on a 2x2x2 object; circular (4 views) or a
    helix (zmax 2, rps 4, vtab 2, fps 16); analytic answer coneBeamSphere.m."""
    if scan == "circle":
        p = G.cone_para(N, N, N, nd, nd, 4, L=(2, 2, 2))
        h = 0.0
    else:
        p = G.cone_para(N, N, N, nd, nd, 0, L=(2, 2, 2), scan="helix", zmax=2, rps=4, vtab=2,
                        fps=16)
        h = 2 / (2 * np.pi * 4)
    x = PH.unit_ball(N, 3).reshape(-1)
    ydet = p["y_det"] * float(p["scale"])
    zdet = p["z_det"] * float(p["scale"])
    Z, Y = np.meshgrid(zdet, ydet, indexing="ij")
    T = p["sd_phi"].astype(np.float64)[:, None, None]
    ex = PH.cone_ball_chord(T, Y[None], Z[None], 0, h, 5.0, 5.0).reshape(-1)
    exn = PH.cone_ball_chord(T, Y[None], Z[None], 0, h, 5.0, 5.0, normalized=True).reshape(-1)
    return p, x, ex, exn


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
