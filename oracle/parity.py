"""Parity of a projector pair at a configuration's own size (test infrastructure).

TEST INFRASTRUCTURE ONLY: used by ``tests/`` and by the parity leg of
``bench.py`` as the checker of GPU results. It never runs on the product path.

The GPU side is passed in as two callables on host arrays, ``forward(x) -> y``
and ``adjoint(y) -> x`` (full sinogram / full volume, FP32). Three numbers are
reported for each operator, as relative L2 errors over the sampled entries:

* ``matched_vs_fp64``: the GPU result against the FP64 exact Siddon model
  (exact intersection lengths of the same rays);
* ``reference_vs_fp64``: the reference's own FP32 CPU kernel against the same
  FP64 model (``Ax_*_mf_cpu_siddon`` forward, ``Atx_*_mf_cpu_new`` chord
  backprojector), i.e. the reference's own error;
* ``matched_vs_reference``: the GPU result against the reference kernel.

The fan is checked in full. A cone volume is checked on seeded random
subsets: the forward on a set of rays, the backprojection on a set of voxels,
each subset value computed by the oracle exactly as the full function would
(``tests/test_oracle_pin.py`` pins the subset functions to the full ones).
Two sinograms feed the backprojectors: the GPU forward projection of the
phantom (the sinogram a reconstruction sees) and N(0, 1) noise (every matrix
entry's error shows, none averages out).

A plan that uses the half or quarter turn (G = 2 or 4 views per walk) defines
view v + j nv/G as view v turned by exactly j 2 pi / G (with the reflection,
G = 8, also view j nv/4 - v as view v reflected about the x axis and turned). FP32 source angles
single(2 pi k / nv) are not exact turns of each other (up to 2.4e-7 rad
apart), so such a plan projects a scan whose angles are snapped to exact
turns. ``snapped(para, G)`` is that scan for the FP64 model (FP64 angles
phi_v + j 2 pi / G); ``matched_vs_fp64_snapped`` measures the kernels'
arithmetic on their own geometry, ``matched_vs_fp64`` includes the snap.
"""
from __future__ import annotations

import os

import numpy as np

from . import (cone_adj_vox, cone_siddon_rays, exact_adjoint, exact_adjoint_vox,
               exact_forward, exact_forward_rays, fan_adj_f32, fan_siddon_f32)


def rel(a, b) -> float:
    a = np.asarray(a, np.float64).reshape(-1)
    b = np.asarray(b, np.float64).reshape(-1)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _three(gpu, ref, exact, exact_snapped=None) -> dict:
    out = {"matched_vs_fp64": rel(gpu, exact), "reference_vs_fp64": rel(ref, exact),
           "matched_vs_reference": rel(gpu, ref)}
    if exact_snapped is not None:
        out["matched_vs_fp64_snapped"] = rel(gpu, exact_snapped)
    return out


def snapped(para, turns: int, reflect: bool = False) -> dict:
    """The scan a plan with `turns` views per rotation orbit projects: FP64
    angles phi[v + j nv/turns] = phi[v] + j 2 pi / turns for v < nv/turns (the
    FP32 angles of the walked views, turned exactly). With the reflection
    about the x axis (reflect, or turns = 8 for the quarter turns with it;
    turns = 1 for a fan's reflection alone, odd nv), the walked views are
    v = 0 .. floor(nv / (2 turns)) -- the last one at exactly pi/turns where
    it is its own mirror image (nv a multiple of 2 turns) -- and view
    j nv/turns - v is view v reflected and turned, at angle
    j 2 pi / turns - phi[v]."""
    if turns == 8:
        turns, reflect = 4, True
    if turns <= 1 and not reflect:
        return para
    turns = max(turns, 1)
    phi = np.asarray(para["sd_phi"], np.float32).astype(np.float64)
    nv = phi.size
    q = nv // turns
    if reflect:
        ov = q // 2
        base = phi[:ov + 1].copy()
        if q % 2 == 0:
            base[ov] = np.pi / turns                  # the end view, its own mirror image
        u = np.arange(nv)
        j, r = u // q, u % q
        refl = r > ov
        vv = np.where(refl, q - r, r)
        step = 2.0 * np.pi / turns
        p64 = np.where(refl, (j + 1) * step - base[vv], base[vv] + j * step)
    else:
        p64 = np.concatenate([phi[:q] + j * (2.0 * np.pi / turns) for j in range(turns)])
    out = dict(para)
    out["phi64"] = p64
    return out


def _threads(threads):
    return threads or max(1, os.cpu_count() or 1)


def fan_parity(para, x, forward, adjoint, seed=0, threads=None, turns=1,
               reflect=False) -> dict:
    """Full fan-beam check: every ray, every pixel."""
    t = _threads(threads)
    ps = snapped(para, turns, reflect) if (turns > 1 or reflect) else None
    x = np.ascontiguousarray(x, np.float32).reshape(-1)
    y = np.asarray(forward(x), np.float32).reshape(-1)
    out = {"forward": dict(rays=int(y.size), **_three(
        y, fan_siddon_f32(x, para, threads=t), exact_forward(x, para, threads=t),
        exact_forward(x, ps, threads=t) if ps else None))}
    rng = np.random.default_rng(seed)
    for name, sino in (("phantom", y), ("random", rng.standard_normal(y.size).astype(np.float32))):
        xa = np.asarray(adjoint(sino), np.float32).reshape(-1)
        out[f"adjoint_{name}_sino"] = dict(voxels=int(xa.size), **_three(
            xa, fan_adj_f32(sino, para, threads=t), exact_adjoint(sino, para, threads=t),
            exact_adjoint(sino, ps, threads=t) if ps else None))
    return out


def cone_parity(para, x, forward, adjoint, n_rays=20000, n_vox=4000, seed=0,
                threads=None, turns=1, reflect=False) -> dict:
    """Cone-beam check on ``n_rays`` random rays and ``n_vox`` random voxels."""
    t = _threads(threads)
    ps = snapped(para, turns, reflect) if (turns > 1 or reflect) else None
    rng = np.random.default_rng(seed)
    x = np.ascontiguousarray(x, np.float32).reshape(-1)
    y = np.asarray(forward(x), np.float32).reshape(-1)
    rays = np.sort(rng.choice(y.size, min(n_rays, y.size), replace=False))
    out = {"forward": dict(rays=int(rays.size), **_three(
        y[rays], cone_siddon_rays(x, para, rays, threads=t),
        exact_forward_rays(x, para, rays, threads=t),
        exact_forward_rays(x, ps, rays, threads=t) if ps else None))}
    vox = np.sort(rng.choice(x.size, min(n_vox, x.size), replace=False))
    for name in ("phantom", "random"):
        sino = y if name == "phantom" else rng.standard_normal(y.size).astype(np.float32)
        xa = np.asarray(adjoint(sino), np.float32).reshape(-1)
        out[f"adjoint_{name}_sino"] = dict(voxels=int(vox.size), **_three(
            xa[vox], cone_adj_vox(sino, para, vox, threads=t),
            exact_adjoint_vox(sino, para, vox, threads=t),
            exact_adjoint_vox(sino, ps, vox, threads=t) if ps else None))
        del sino
    return out
