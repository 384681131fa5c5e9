"""Seeded synthetic objects and analytic projections used as known answers.

Arrays are C-ordered ``(ny, nx)`` / ``(nz, ny, nx)`` so the flat index is the
reference's ``iz*ny*nx + iy*nx + ix`` (x fastest). Coordinates are normalised
to ``[-1, 1]`` per axis at voxel centres, like ``unitBall.m:3-4``.
"""
from __future__ import annotations

import numpy as np


def _centres(n: int) -> np.ndarray:
    return (2.0 / n) * (np.arange(n) - n / 2 + 0.5)


def ellipses_2d(n: int, seed: int = 0, count: int = 10) -> np.ndarray:
    """Sum of ``count`` random ellipses: centres U[-0.8,0.8]^2, semi-axes
    U[0.05,0.5], angle U[0,pi], intensity U[0.1,1.0] (additive)."""
    rng = np.random.default_rng(seed)
    c = _centres(n)
    Y, X = np.meshgrid(c, c, indexing="ij")
    img = np.zeros((n, n), np.float64)
    for _ in range(count):
        cx, cy = rng.uniform(-0.8, 0.8, 2)
        a, b = rng.uniform(0.05, 0.5, 2)
        th = rng.uniform(0, np.pi)
        val = rng.uniform(0.1, 1.0)
        xr = (X - cx) * np.cos(th) + (Y - cy) * np.sin(th)
        yr = -(X - cx) * np.sin(th) + (Y - cy) * np.cos(th)
        img[(xr / a) ** 2 + (yr / b) ** 2 <= 1.0] += val
    return img.astype(np.float32)


def ellipsoids_3d(n: int, seed: int = 0, count: int = 12, nz: int | None = None,
                  chunk: int = 32) -> np.ndarray:
    """Sum of ``count`` random ellipsoids, same distributions as ellipses_2d,
    each rotated about z by a random angle. Built slab by slab so 512^3 fits."""
    rng = np.random.default_rng(seed)
    nz = n if nz is None else nz
    params = []
    for _ in range(count):
        cx, cy, cz = rng.uniform(-0.8, 0.8, 3)
        a, b, cc = rng.uniform(0.05, 0.5, 3)
        th = rng.uniform(0, np.pi)
        val = rng.uniform(0.1, 1.0)
        params.append((cx, cy, cz, a, b, cc, np.cos(th), np.sin(th), val))
    c = _centres(n).astype(np.float32)
    cz_all = _centres(nz).astype(np.float32)
    Y, X = np.meshgrid(c, c, indexing="ij")
    vol = np.zeros((nz, n, n), np.float32)
    for z0 in range(0, nz, chunk):
        zs = cz_all[z0:z0 + chunk][:, None, None]
        slab = vol[z0:z0 + chunk]
        for (cx, cy, cz, a, b, cc, ct, st, val) in params:
            if np.all(np.abs(zs - cz) > cc):
                continue
            xr = (X - cx) * ct + (Y - cy) * st
            yr = -(X - cx) * st + (Y - cy) * ct
            inside = (xr / a) ** 2 + (yr / b) ** 2 + ((zs - cz) / cc) ** 2 <= 1.0
            slab += np.float32(val) * inside
    return vol


def unit_ball(n: int, d: int) -> np.ndarray:
    """Indicator of the unit disc/ball sampled at voxel centres (unitBall.m:1-33)."""
    c = _centres(n)
    if d == 2:
        Y, X = np.meshgrid(c, c, indexing="ij")
        return (np.sqrt(X ** 2 + Y ** 2) <= 1).astype(np.float32)
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    return (np.sqrt(X ** 2 + Y ** 2 + Z ** 2) <= 1).astype(np.float32)


def fan_disc_chord(a, SO, OD):
    """Chord of the unit disc along the fan ray to flat-detector offset ``a``
    (testBall.m:13, generalised): 2*sqrt(1 - d^2), d = SO|a|/sqrt(SD^2 + a^2)."""
    a = np.asarray(a, np.float64)
    SD = SO + OD
    d = SO * np.abs(a) / np.sqrt(SD ** 2 + a ** 2)
    return np.where(d < 1, 2 * np.sqrt(np.clip(1 - d ** 2, 0, None)), 0.0)


def cone_ball_chord(t, a, b, zeta, h, Rs, Rd, normalized=False):
    """Cone-beam transform of the unit ball (coneBeamSphere.m:10-16): source
    angle t, detector coordinates (a, b), axial shift zeta, helix h = P/2pi."""
    t, a, b = (np.asarray(v, np.float64) for v in (t, a, b))
    R = Rs + Rd
    zs = h * t + zeta
    disc = (Rs * R - b * zs) ** 2 - (a ** 2 + b ** 2 + R ** 2) * (Rs ** 2 + (zs + 1) * (zs - 1))
    den = a ** 2 + b ** 2 + R ** 2
    ok = disc >= 0
    root = np.sqrt(np.where(ok, disc, 0.0))
    y = 2 * root / den if normalized else 2 * np.sqrt(np.where(ok, disc, 0.0) / den)
    return np.where(ok, y, 0.0)
