"""The ``para`` fields of geometry.py follow setPara.m's rounding order.

MATLAB evaluates each operation by its operands' classes: single with single
in single precision; an operation with one double operand in double, its
result rounded to single. The scanner's SO, OD, Ly, Lz and y_os are single
properties (FanBeamScanner.m:5-10, ConeBeamScanner.m:10-16); the counts na,
nb, nd and the helix step h are double. Each expected value below is written
out step by step from the cited setPara.m line, at pitches that do not divide
evenly (Ly = 2*sqrt(2)*L, odd detector counts), so a wrong rounding order
shows as a differing bit.
"""
import math

import numpy as np

from framelab_gb300 import geometry as G

f32, f64 = np.float32, np.float64


def test_fan_fields_follow_setpara_order():
    L, n, nd, nv = 1.0, 256, 511, 360
    Ly = 2 * math.sqrt(2.0) * L
    p = G.fan_para(n, n, nd, nv, L=(L, L), SO=500.0, OD=500.0, Ly=Ly)
    scale = f32(L / n)                                  # setPara.m:5 single(Dx(1))
    assert p["scale"] == scale
    assert p["SO"] == f32(f32(500.0) / scale)           # setPara.m:8 single / single
    dy = f32(f64(f32(Ly)) / f64(nd))                    # setPara.m:10 single / double
    assert p["dy_det"] == f32(dy / scale)               # setPara.m:11 single / single
    # setPara.m:23: ((-nd/2:nd/2-1)+0.5) is double; times the single dy_det
    # is one double product rounded to single; + y_os (single) is single;
    # / scale is single
    k = -nd / 2.0 + np.arange(nd) + 0.5
    want = ((k * f64(dy)).astype(f32) + f32(0.0)).astype(f32) / scale
    assert np.array_equal(p["y_det"], want.astype(f32))
    # setPara.m:22: single(2*pi/nv*(0:nv-1)) -- double, rounded once
    assert np.array_equal(p["sd_phi"], (2 * math.pi / nv * np.arange(nv)).astype(f32))


def test_cone_fields_follow_setpara_order():
    n, na, nb, nv = 64, 97, 75, 90
    L = (n * 0.7, n * 0.7, n * 0.7)
    Ly, Lz = 2 * math.sqrt(2.0) * 30.0, math.pi * 20.0
    p = G.cone_para(n, n, n, na, nb, nv, L=L, SO=600.0, OD=600.0, Ly=Ly, Lz=Lz, y_os=0.3)
    scale = f32(L[0] / n)
    dy = f32(f64(f32(Ly)) / f64(na))                    # setPara.m:10
    dz = f32(f64(f32(Lz)) / f64(nb))                    # setPara.m:11
    assert p["dy_det"] == f32(dy / scale)               # setPara.m:12
    assert p["dz_det"] == f32(dz / scale)               # setPara.m:13
    assert p["y_os"] == f32(f32(0.3) / f32(dy / scale))  # setPara.m:14 single / single
    assert p["dz"] == f32(f32(L[2] / n) / scale)        # setPara.m:22
    ka = -na / 2.0 + np.arange(na) + 0.5
    kb = -nb / 2.0 + np.arange(nb) + 0.5
    # setPara.m:53-54 (the single y_os property is added in single)
    assert np.array_equal(p["y_det"], (((ka * f64(dy)).astype(f32) + f32(0.3)) / scale).astype(f32))
    assert np.array_equal(p["z_det"], ((kb * f64(dz)).astype(f32) / scale).astype(f32))


def test_helix_sd_z_is_a_double_product():
    zmax, rps, vtab, fps = 1.0, 1.0, 1.0, 16.0
    p = G.cone_para(32, 32, 32, 48, 40, L=(2, 2, 2), scan="helix", zmax=zmax, rps=rps,
                    vtab=vtab, fps=fps)
    scale = p["scale"]
    phi_max = rps * zmax * 2 * math.pi / vtab
    dphi = 2 * math.pi * rps / fps
    base = -phi_max / 2 + dphi * np.arange(int(math.floor(phi_max / dphi + 1e-10)) + 1)
    sd_phi = base.astype(f32)                            # setPara.m:32
    assert np.array_equal(p["sd_phi"], sd_phi)
    h = vtab / (2 * math.pi * rps)
    # setPara.m:35: single(h*sd_phi)/scale -- double h times single sd_phi is
    # a double product rounded to single, then a single division
    want = ((h * sd_phi.astype(f64)).astype(f32) / scale).astype(f32)
    assert np.array_equal(p["sd_z"], want)
    # and it is not the product formed in single (h rounded first) everywhere
    single = ((f32(h) * sd_phi).astype(f32) / scale).astype(f32)
    assert not np.array_equal(want, single)


def test_multi_helix_sd_z_is_rounded_once():
    kw = dict(scan="multiHelix", zmax=1.0, rps=1.0, vtab=1.0, fps=16.0, n_helix=2,
              phase_shift=(0.0, 1.0))
    p = G.cone_para(32, 32, 32, 48, 40, L=(2, 2, 2), **kw)
    scale = p["scale"]
    phi_max = 2 * math.pi
    dphi = 2 * math.pi / 16.0
    base = -phi_max / 2 + dphi * np.arange(17)
    h = 1.0 / (2 * math.pi)
    one = ((h * base).astype(f32) / scale).astype(f32)   # setPara.m:49
    assert np.array_equal(p["sd_z"], np.concatenate([one, one]))
    assert np.array_equal(p["sd_phi"], np.concatenate([base.astype(f32),
                                                       (base + 1.0).astype(f32)]))
