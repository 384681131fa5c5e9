"""Pins the oracle restatement against the reference's own CPU kernels.

The reference sources (compiled unmodified into oracle/_ref) are only present
where the reference checkout exists; elsewhere the committed fixtures in
tests/golden/ (generated from oracle/_ref by tests/golden/make_golden.py) pin
the restatement instead.
"""
import glob
import os

import numpy as np
import pytest

import oracle as O
from framelab_gb300 import geometry as G

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
need_ref = pytest.mark.skipif(not O.have_ref(), reason="reference sources not built here")


def _rand_fan(rng, n, nd, nv):
    return G.fan_para(n, n, nd, nv, L=(2, 2), SO=rng.uniform(2, 6), OD=rng.uniform(2, 6),
                      Ly=rng.uniform(3, 8))


def _rand_cone(rng, n, na, nb, nv, scan="circle"):
    kw = {}
    if scan != "circle":
        kw = dict(scan=scan, zmax=0.5, rps=1.0, vtab=1.0, fps=max(nv, 4))
    return G.cone_para(n, n, n, na, nb, nv, L=(2, 2, 2), SO=rng.uniform(3, 6),
                       OD=rng.uniform(3, 6), Ly=rng.uniform(3, 8), Lz=rng.uniform(3, 8), **kw)


@need_ref
@pytest.mark.parametrize("seed", range(8))
def test_fan_restatement_is_bit_exact(seed):
    rng = np.random.default_rng(seed)
    n = [8, 16, 32, 64][seed % 4]
    p = _rand_fan(rng, n, [12, 24, 50, 33][seed % 4], [5, 7, 16][seed % 3])
    X = rng.standard_normal(n * n).astype(np.float32)
    assert np.array_equal(O.fan_siddon_f32(X, p), O.ref_fan_siddon(X, p))
    assert np.array_equal(O.fan_gao_f32(X, p), O.ref_fan_new(X, p))
    Y = rng.standard_normal(len(p["y_det"]) * len(p["sd_phi"])).astype(np.float32)
    assert np.array_equal(O.fan_adj_f32(Y, p), O.ref_fan_adj(Y, p))


@need_ref
@pytest.mark.parametrize("seed", range(6))
def test_cone_restatement_is_bit_exact(seed):
    rng = np.random.default_rng(100 + seed)
    n = [8, 16, 24][seed % 3]
    scan = "helix" if seed % 2 else "circle"
    p = _rand_cone(rng, n, [12, 20][seed % 2], [10, 14][seed % 2], [3, 5, 9][seed % 3], scan)
    X = rng.standard_normal(n ** 3).astype(np.float32)
    assert np.array_equal(O.cone_siddon_f32(X, p), O.ref_cone_siddon(X, p))
    (a, an), (b, bn) = O.cone_gao_f32(X, p), O.ref_cone_new(X, p)
    assert np.array_equal(a, b) and np.array_equal(an, bn)
    Y = rng.standard_normal(len(p["y_det"]) * len(p["z_det"]) * len(p["sd_phi"])).astype(np.float32)
    assert np.array_equal(O.cone_adj_f32(Y, p), O.ref_cone_adj(Y, p))


@need_ref
@pytest.mark.parametrize("seed", range(8))
def test_fan_finite_beam_restatement_is_bit_exact(seed):
    rng = np.random.default_rng(200 + seed)
    n = [8, 16, 32, 40][seed % 4]
    p = _rand_fan(rng, n, [12, 24, 50, 33][seed % 4], [5, 7, 16][seed % 3])
    if seed % 2:                       # an offset detector and arbitrary angles
        p = G.fan_para(n, n, len(p["y_det"]), 9, L=(2, 2), SO=3.5, OD=4.0, Ly=5.0,
                       y_os=0.37, sd_phi=rng.uniform(-4, 4, 9))
    X = rng.standard_normal(n * n).astype(np.float32)
    assert np.array_equal(O.fan_fb_f32(X, p), O.ref_fan_fb(X, p))
    Y = rng.standard_normal(len(p["y_det"]) * len(p["sd_phi"])).astype(np.float32)
    assert np.array_equal(O.fan_fb_adj_f32(Y, p), O.ref_fan_fb_adj(Y, p))


def _golden_cases():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def test_golden_fixtures_exist():
    assert len(_golden_cases()) >= 4


@pytest.mark.parametrize("path", _golden_cases(), ids=os.path.basename)
def test_restatement_matches_golden(path):
    from tests.golden.fixtures import load_case
    case = load_case(path)
    p, kind = case["para"], case["kind"]
    if kind == "fan_siddon":
        out = O.fan_siddon_f32(case["x"], p)
    elif kind == "fan_adj":
        out = O.fan_adj_f32(case["x"], p)
    elif kind == "cone_siddon":
        out = O.cone_siddon_f32(case["x"], p)
    elif kind == "cone_adj":
        out = O.cone_adj_f32(case["x"], p)
    elif kind == "fan_new":
        out = O.fan_gao_f32(case["x"], p)
    elif kind == "fan_fb":
        out = O.fan_fb_f32(case["x"], p)
    elif kind == "fan_fb_adj":
        out = O.fan_fb_adj_f32(case["x"], p)
    elif kind == "cone_new":
        out, yn = O.cone_gao_f32(case["x"], p)
        assert np.array_equal(yn, case["extra"]["yNorm"])
    else:
        pytest.skip(f"no restatement for {kind}")
    assert np.array_equal(out, case["y"]), kind


@pytest.mark.parametrize("scan", ["circle", "helix"])
def test_subset_functions_equal_the_full_ones(scan):
    """The ray- and voxel-subset oracles used for parity at full problem size
    return, at every sampled entry, exactly what the full functions write
    (FP32 restatements bit for bit; the FP64 voxel chord sum to FP64
    rounding against the FP64 Siddon transpose)."""
    rng = np.random.default_rng(11)
    p = _rand_cone(rng, 20, 36, 28, 10, scan)
    X = rng.standard_normal(20 ** 3).astype(np.float32)
    y = O.cone_siddon_f32(X, p)
    rays = rng.choice(y.size, 400, replace=False)
    assert np.array_equal(O.cone_siddon_rays(X, p, rays, threads=2), y[rays])
    e = O.exact_forward(X, p)
    assert np.array_equal(O.exact_forward_rays(X, p, rays, threads=2), e[rays])
    Y = rng.standard_normal(y.size).astype(np.float32)
    vox = rng.choice(X.size, 300, replace=False)
    assert np.array_equal(O.cone_adj_vox(Y, p, vox, threads=2), O.cone_adj_f32(Y, p)[vox])
    ea = O.exact_adjoint(Y, p)
    got = O.exact_adjoint_vox(Y, p, vox, threads=2)
    assert np.max(np.abs(got - ea[vox])) <= 1e-12 * np.max(np.abs(ea))
