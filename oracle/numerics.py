"""FP64 numpy restatement of FrameLab's solver-side algebra (test infrastructure).

Only tests/ and bench.py's CPU baseline use this module; the product library
never does.

* framelet analysis/synthesis follow GenerateFrameletFilter.m:9-17,
  ConvSymAsym3D.m:18-34 (imfilter 'circular' = circular correlation, 'same',
  centred), FraDecMultiLevel3D.m:14-47 and FraRecMultiLevel3D.m:14-48;
* soft-thresholding follows softThreshold.m:47-80 (every subband except the
  low-pass (1,1,1) of each level);
* CGLS follows solveCGLS.m:6-31, split Bregman solveSplitBregman.m:15-41
  (with v = v + (Wu - alpha), i.e. the class, not testTWFRecon.m).

Array layout: C order (nz, ny, nx) -- x fastest, like MATLAB's (nx, ny, nz).
MATLAB dim 1 = x = numpy axis -1, dim 2 = y = axis -2, dim 3 = z = axis -3.
"""
from __future__ import annotations

import numpy as np

SQ2 = np.sqrt(2.0)
# decomposition filters D{1..3} and reconstruction filters R{1..3} (linear)
LINEAR_D = [np.array([1, 2, 1]) / 4, -np.array([1, 0, -1]) / 4 * SQ2, np.array([-1, 2, -1]) / 4]
LINEAR_R = [np.array([1, 2, 1]) / 4, -np.array([-1, 0, 1]) / 4 * SQ2, np.array([-1, 2, -1]) / 4]
HAAR_D = [np.array([0, 1, 1]) / 2, -np.array([0, 1, -1]) / 2]
HAAR_R = [np.array([1, 1, 0]) / 2, -np.array([-1, 1, 0]) / 2]
SQ6 = np.sqrt(6.0)
CUBIC_D = [np.array([1, 4, 6, 4, 1]) / 16, -np.array([1, 2, 0, -2, -1]) / 8,
           np.array([-1, 0, 2, 0, -1]) / 16 * SQ6, np.array([-1, 2, 0, -2, 1]) / 8,
           -np.array([1, -4, 6, -4, 1]) / 16]
CUBIC_R = [np.array([1, 4, 6, 4, 1]) / 16, -np.array([-1, -2, 0, 2, 1]) / 8,
           np.array([-1, 0, 2, 0, -1]) / 16 * SQ6, np.array([1, -2, 0, 2, -1]) / 8,
           -np.array([1, -4, 6, -4, 1]) / 16]


def filters(kind="linear"):
    return {"linear": (LINEAR_D, LINEAR_R), "haar": (HAAR_D, HAAR_R),
            "cubic": (CUBIC_D, CUBIC_R)}[kind]


def corr_circ(a, m, axis, level):
    """C = imfilter(A, ker, 'circular') along `axis` with ker = M dilated by 2^(L-1):
    C[i] = sum_k m[k] * A[i + (k - c) * step], c = (len(m)-1)/2."""
    step = 2 ** (level - 1)
    c = (len(m) - 1) // 2
    out = np.zeros_like(a, dtype=np.float64)
    for k, mk in enumerate(m):
        if mk == 0:
            continue
        out += mk * np.roll(a, -(k - c) * step, axis=axis)
    return out


def frame_dec_level(a, D, level):
    """One level of FraDec3D: subband (i,j,k) = D_i along y, D_j along x, D_k along z."""
    a = np.asarray(a, np.float64)
    nd = len(D)
    out = {}
    for i in range(nd):
        ti = corr_circ(a, D[i], -2, level)
        for j in range(nd):
            tj = corr_circ(ti, D[j], -1, level)
            for k in range(nd):
                out[(i, j, k)] = corr_circ(tj, D[k], -3, level)
    return out


def frame_rec_level(c, R, level):
    """One level of FraRec3D: sum over subbands of the R-filtered coefficients."""
    nr = len(R)
    shape = c[(0, 0, 0)].shape
    rec = np.zeros(shape)
    for i in range(nr):
        t1 = np.zeros(shape)
        for j in range(nr):
            t2 = np.zeros(shape)
            for k in range(nr):
                t2 += corr_circ(c[(i, j, k)], R[k], -3, level)
            t1 += corr_circ(t2, R[j], -1, level)
        rec += corr_circ(t1, R[i], -2, level)
    return rec


def frame_dec(a, levels=2, kind="linear"):
    """FraDecMultiLevel3D: level k+1 decomposes the low-pass of level k."""
    D, _ = filters(kind)
    out = []
    cur = np.asarray(a, np.float64)
    for lev in range(1, levels + 1):
        d = frame_dec_level(cur, D, lev)
        out.append(d)
        cur = d[(0, 0, 0)]
    return out


def frame_rec(coefs, kind="linear"):
    """FraRecMultiLevel3D: the low-pass of level k-1 is replaced by the
    reconstruction of level k."""
    _, R = filters(kind)
    c = [dict(x) for x in coefs]
    L = len(c)
    for k in range(L, 1, -1):
        c[k - 2][(0, 0, 0)] = frame_rec_level(c[k - 1], R, k)
    return frame_rec_level(c[0], R, 1)


def shrink(coefs, tau):
    """softThreshold.m:65-78: sign(a)*max(|a|-tau, 0) except band (1,1,1) of each level."""
    out = []
    for lev in coefs:
        d = {}
        for key, a in lev.items():
            d[key] = a if key == (0, 0, 0) else np.sign(a) * np.maximum(np.abs(a) - tau, 0.0)
        out.append(d)
    return out


def coef_add(a, b, sa=1.0, sb=1.0):
    return [{k: sa * x[k] + sb * y[k] for k in x} for x, y in zip(a, b)]


def cgls(apply_normal, b, u0, lam, iters, tol=1e-14):
    """solveCGLS.m:6-31 in FP64. apply_normal(x) returns A^T A x."""
    A_loc = lambda x: apply_normal(x) + lam * x  # noqa: E731
    r = A_loc(u0) - b
    p = -r
    u = u0.copy()
    gamma = float(np.dot(r, r))
    hist = []
    for _ in range(iters):
        q = A_loc(p)
        alpha = gamma / float(np.dot(p, q))
        u = u + alpha * p
        r = r + alpha * q
        gnew = float(np.dot(r, r))
        beta = gnew / gamma
        p = -r + beta * p
        gamma = gnew
        hist.append(gnew)
        if gamma < tol:
            break
    return u, hist


def split_bregman(A, At, W, Wt, f, u0, lam, mu, outer, cg_iters, cg_tol=1e-10):
    """solveSplitBregman.m:15-41 (v = v + (Wu - alpha)); W returns a coefficient
    list, Wt maps it back. u0, f flat FP64 vectors."""
    alpha = W(u0)
    v = [dict(x) for x in alpha]
    Atf = At(f)
    b = Atf + mu * Wt(coef_add(alpha, v, 1.0, -1.0))
    u = u0.copy()
    normal = lambda x: At(A(x))  # noqa: E731
    for _ in range(outer):
        u, _h = cgls(normal, b, u, mu, cg_iters, cg_tol)
        Wu = W(u)
        alpha = shrink(coef_add(v, Wu), lam / mu)
        v = coef_add(v, coef_add(Wu, alpha, 1.0, -1.0))
        b = Atf + mu * Wt(coef_add(alpha, v, 1.0, -1.0))
    return u
