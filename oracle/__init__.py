"""CPU checker for the FrameLab-GB300 hot path.

TEST INFRASTRUCTURE ONLY. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this package, and only as the thing the
GPU results are checked against or timed beside. The product library
(``framelab_gb300``) never imports, loads or calls anything here.

Contents:
  * ``liboracle.so`` (oracle.c): a C restatement of the reference's
    single-precision CPU kernels (bit-exact), and an FP64 exact Siddon model.
  * ``_ref/liboracle_ref.so``: the reference's own CPU kernels compiled
    unmodified (Makefile); present only where the reference checkout exists.
  * ``numerics.py``: FP64 numpy restatement of the framelet transform,
    soft-shrink, CGLS and split Bregman.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(HERE, "liboracle.so")
_REFLIB = os.path.join(HERE, "_ref", "liboracle_ref.so")
_lock = threading.Lock()
_libs = {}

fp = C.POINTER(C.c_float)
dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
i64p = C.POINTER(C.c_int64)


def build(with_ref: bool = True) -> None:
    """Compile liboracle.so (and _ref when the reference sources exist)."""
    target = "all" if with_ref else "liboracle.so"
    subprocess.run(["make", "-s", "-C", HERE, target], check=True)


def _load(path, name):
    with _lock:
        if name not in _libs:
            if not os.path.exists(path):
                if name == "oracle":
                    build(with_ref=False)
                else:
                    return None
            _libs[name] = C.CDLL(path)
        return _libs[name]


def lib():
    return _load(_LIB, "oracle")


def ref_lib():
    """The reference's own CPU kernels, or None where they were not built."""
    return _load(_REFLIB, "ref")


def have_ref() -> bool:
    return os.path.exists(_REFLIB)


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(np.asarray(a).astype(np.int32))


def P(a):
    if a.dtype == np.float32:
        return a.ctypes.data_as(fp)
    if a.dtype == np.float64:
        return a.ctypes.data_as(dp)
    if a.dtype == np.int64:
        return a.ctypes.data_as(i64p)
    return a.ctypes.data_as(ip)


F, I, D = C.c_float, C.c_int, C.c_double


def _split(n, parts):
    parts = max(1, min(parts, n))
    b = np.linspace(0, n, parts + 1).astype(int)
    return [(int(b[k]), int(b[k + 1])) for k in range(parts) if b[k + 1] > b[k]]


def _run(fn, ranges, threads):
    if threads <= 1 or len(ranges) == 1:
        for r in ranges:
            fn(*r)
        return
    with ThreadPoolExecutor(threads) as ex:  # ctypes releases the GIL
        list(ex.map(lambda r: fn(*r), ranges))


# --------------------------------------------------------------------------
# FP32 restatement (bit-exact with the reference's CPU kernels)
# --------------------------------------------------------------------------

def fan_siddon_f32(X, p, threads=1, views=None):
    """Ax_fan_mf_cpu_siddon (Ax_fan_mf_cpu_siddon.cpp:19-93), views [v0, v1)."""
    L = lib()
    X = _f(X); sd = _f(p["sd_phi"]); yd = _f(p["y_det"]); idx = _i(p["id_X"])
    nv, nd = len(sd), len(yd)
    v0, v1 = views or (0, nv)
    y = np.zeros(nv * nd, np.float32)

    def go(a, b):
        L.orc_fan_siddon_f32(P(X), P(y), F(p["SO"]), F(p["OD"]), F(p["scale"]),
                             I(int(p["nx"])), I(int(p["ny"])), I(a), I(b), P(sd), I(nd),
                             P(yd), P(idx))
    rng = [(v0 + a, v0 + b) for a, b in _split(v1 - v0, threads * 4 if threads > 1 else 1)]
    _run(go, rng, threads)
    return y


def cone_siddon_f32(X, p, threads=1, views=None):
    """Ax_cone_mf_cpu_siddon (Ax_cone_mf_cpu_siddon.cpp:19-134), views [v0, v1)."""
    L = lib()
    X = _f(X); sd = _f(p["sd_phi"]); sz = _f(p["sd_z"]); yd = _f(p["y_det"])
    zd = _f(p["z_det"]); idx = _i(p["id_X"])
    nv, na, nb = len(sd), len(yd), len(zd)
    v0, v1 = views or (0, nv)
    y = np.zeros(nv * na * nb, np.float32)

    def go(a, b):
        L.orc_cone_siddon_f32(P(X), P(y), F(p["SO"]), F(p["OD"]), F(p["scale"]),
                              I(int(p["nx"])), I(int(p["ny"])), I(int(p["nz"])), I(a), I(b),
                              P(sd), P(sz), I(na), I(nb), P(yd), P(zd), P(idx), F(p["dz"]))
    rng = [(v0 + a, v0 + b) for a, b in _split(v1 - v0, threads * 4 if threads > 1 else 1)]
    _run(go, rng, threads)
    return y


def fan_adj_f32(Y, p, threads=1, rows=None):
    """Atx_fan_mf_cpu_new (Atx_fan_mf_cpu_new.cpp:21-63), image rows [r0, r1)."""
    L = lib()
    Y = _f(Y); cp = _f(p["cos_phi"]); sp = _f(p["sin_phi"]); cd = _f(p["cos_det"])
    sdt = _f(p["sin_det"]); idY = _i(np.asarray(p["id_Y"]).T.reshape(-1)); Nv = _i(p["Nv"])
    nx, ny, nt = int(p["nx"]), int(p["ny"]), int(p["nt"])
    nd = len(p["y_det"])
    x = np.zeros(nx * ny * nt, np.float32)
    r0, r1 = rows or (0, ny)

    def go(a, b):
        L.orc_fan_adj_f32(P(x), P(Y), F(p["SO"]), F(p["OD"]), F(p["scale"]), I(nx), I(ny),
                          I(nd), F(p["dy_det"]), F(p["y_os"]), I(nt), P(idY), P(Nv),
                          I(int(p["tmp_size"])), P(cp), P(sp), P(cd), P(sdt), I(a), I(b))
    rng = [(r0 + a, r0 + b) for a, b in _split(r1 - r0, threads * 4 if threads > 1 else 1)]
    _run(go, rng, threads)
    return x


def cone_adj_f32(Y, p, threads=1, slices=None):
    """Atx_cone_mf_cpu_new (Atx_cone_mf_cpu_new.cpp:23-85), slices [z0, z1)."""
    L = lib()
    Y = _f(Y); cp = _f(p["cos_phi"]); sp = _f(p["sin_phi"]); sz = _f(p["sd_z"])
    yd = _f(p["y_det"]); zd = _f(p["z_det"]); idY = _i(np.asarray(p["id_Y"]).T.reshape(-1))
    Nv = _i(p["Nv"])
    nx, ny, nz, nt = int(p["nx"]), int(p["ny"]), int(p["nz"]), int(p["nt"])
    na, nb = len(yd), len(zd)
    x = np.zeros(nx * ny * nz * nt, np.float32)
    z0, z1 = slices or (0, nz)

    def go(a, b):
        L.orc_cone_adj_f32(P(x), P(Y), F(p["SO"]), F(p["OD"]), F(p["scale"]), I(nx), I(ny),
                           I(nz), P(sz), P(yd), P(zd), F(p["dy_det"]), F(p["y_os"]),
                           F(p["dz_det"]), F(p["dz"]), I(nt), P(idY), P(Nv),
                           I(int(p["tmp_size"])), P(cp), P(sp), I(na), I(nb), I(a), I(b))
    rng = [(z0 + a, z0 + b) for a, b in _split(z1 - z0, threads * 4 if threads > 1 else 1)]
    _run(go, rng, threads)
    return x


# --------------------------------------------------------------------------
# The reference itself (oracle/_ref), same calling conventions
# --------------------------------------------------------------------------

def _need_ref():
    R = ref_lib()
    if R is None:
        raise RuntimeError("oracle/_ref not built (reference sources absent)")
    return R


def ref_fan_siddon(X, p):
    R = _need_ref()
    X = _f(X); sd = _f(p["sd_phi"]); yd = _f(p["y_det"]); idx = _i(p["id_X"])
    y = np.zeros(len(sd) * len(yd), np.float32)
    R.ref_Ax_fan_mf_cpu_siddon(P(X), P(y), F(p["SO"]), F(p["OD"]), F(p["scale"]),
                               I(int(p["nx"])), I(int(p["ny"])), I(len(sd)), P(sd), I(len(yd)),
                               P(yd), P(idx))
    return y


def ref_fan_new(X, p):
    R = _need_ref()
    X = _f(X); sd = _f(p["sd_phi"]); yd = _f(p["y_det"]); idx = _i(p["id_X"])
    y = np.zeros(len(sd) * len(yd), np.float32)
    R.ref_Ax_fan_mf_cpu_new(P(X), P(y), F(p["SO"]), F(p["OD"]), F(p["scale"]),
                            I(int(p["nx"])), I(int(p["ny"])), I(len(sd)), P(sd), I(len(yd)),
                            P(yd), P(idx))
    return y


def ref_cone_siddon(X, p):
    R = _need_ref()
    X = _f(X); sd = _f(p["sd_phi"]); sz = _f(p["sd_z"]); yd = _f(p["y_det"])
    zd = _f(p["z_det"]); idx = _i(p["id_X"])
    y = np.zeros(len(sd) * len(yd) * len(zd), np.float32)
    R.ref_Ax_cone_mf_cpu_siddon(P(X), P(y), F(p["SO"]), F(p["OD"]), F(p["scale"]),
                                I(int(p["nx"])), I(int(p["ny"])), I(int(p["nz"])), I(len(sd)),
                                P(sd), P(sz), I(len(yd)), I(len(zd)), P(yd), P(zd), P(idx),
                                F(p["dz"]))
    return y


def ref_cone_new(X, p):
    R = _need_ref()
    X = _f(X); sd = _f(p["sd_phi"]); sz = _f(p["sd_z"]); yd = _f(p["y_det"])
    zd = _f(p["z_det"]); idx = _i(p["id_X"])
    n = len(sd) * len(yd) * len(zd)
    y = np.zeros(n, np.float32); yn = np.zeros(n, np.float32)
    R.ref_Ax_cone_mf_cpu_new(P(X), P(y), P(yn), F(p["SO"]), F(p["OD"]), F(p["scale"]),
                             I(int(p["nx"])), I(int(p["ny"])), I(int(p["nz"])), I(len(sd)),
                             P(sd), P(sz), I(len(yd)), I(len(zd)), P(yd), P(zd), P(idx),
                             F(p["dz"]))
    return y, yn


def ref_fan_adj(Y, p):
    R = _need_ref()
    Y = _f(Y); sd = _f(p["sd_phi"]); yd = _f(p["y_det"]); cp = _f(p["cos_phi"])
    sp = _f(p["sin_phi"]); cd = _f(p["cos_det"]); sdt = _f(p["sin_det"])
    idY = _i(np.asarray(p["id_Y"]).T.reshape(-1)); Nv = _i(p["Nv"])
    nx, ny, nt = int(p["nx"]), int(p["ny"]), int(p["nt"])
    x = np.zeros(nx * ny * nt, np.float32)
    R.ref_Atx_fan_mf_cpu_new(P(x), P(Y), F(p["SO"]), F(p["OD"]), F(p["scale"]), I(nx), I(ny),
                             P(sd), I(len(yd)), P(yd), F(p["dy_det"]), F(p["y_os"]), I(nt),
                             P(idY), P(Nv), I(int(p["tmp_size"])), I(int(p["nv"])), P(cp), P(sp),
                             P(cd), P(sdt))
    return x


def ref_cone_adj(Y, p):
    R = _need_ref()
    Y = _f(Y); cp = _f(p["cos_phi"]); sp = _f(p["sin_phi"]); sz = _f(p["sd_z"])
    yd = _f(p["y_det"]); zd = _f(p["z_det"]); idY = _i(np.asarray(p["id_Y"]).T.reshape(-1))
    Nv = _i(p["Nv"])
    nx, ny, nz, nt = int(p["nx"]), int(p["ny"]), int(p["nz"]), int(p["nt"])
    x = np.zeros(nx * ny * nz * nt, np.float32)
    R.ref_Atx_cone_mf_cpu_new(P(x), P(Y), F(p["SO"]), F(p["OD"]), F(p["scale"]), I(nx), I(ny),
                              I(nz), P(sz), P(yd), P(zd), F(p["dy_det"]), F(p["y_os"]),
                              F(p["dz_det"]), F(p["dz"]), I(nt), P(idY), P(Nv),
                              I(int(p["tmp_size"])), I(len(cp)), P(cp), P(sp), I(len(yd)),
                              I(len(zd)))
    return x


# --------------------------------------------------------------------------
# FP64 exact Siddon model
# --------------------------------------------------------------------------

def _exact_args(p):
    """FP64 model inputs: the source angles in FP64 (the FP32 sd_phi, or an
    explicit "phi64" array, e.g. views snapped to exact turns), the other
    geometry as the FP32 para holds it."""
    sd = _d(p["phi64"]) if "phi64" in p else _d(_f(p["sd_phi"]))
    yd = _f(p["y_det"])
    cone = "nz" in p
    sz = _f(p["sd_z"]) if cone else np.zeros(len(sd), np.float32)
    zd = _f(p["z_det"]) if cone else np.zeros(1, np.float32)
    nz = int(p["nz"]) if cone else 1
    dz = float(p["dz"]) if cone else 1.0
    return sd, sz, yd, zd, nz, dz


def exact_forward(X, p, threads=1, views=None):
    """y = scale * sum(len * x) in FP64 for every ray (fan: nz = 1)."""
    L = lib()
    sd, sz, yd, zd, nz, dz = _exact_args(p)
    X = _d(X)
    nv, na, nb = len(sd), len(yd), len(zd)
    v0, v1 = views or (0, nv)
    y = np.zeros(nv * na * nb, np.float64)

    def go(a, b):
        L.orc_exact_forward_f64(P(X), P(y), D(float(p["SO"])), D(float(p["OD"])),
                                D(float(p["scale"])), I(int(p["nx"])), I(int(p["ny"])), I(nz),
                                D(dz), I(a), I(b), P(sd), P(sz), I(na), I(nb), P(yd), P(zd))
    rng = [(v0 + a, v0 + b) for a, b in _split(v1 - v0, threads * 4 if threads > 1 else 1)]
    _run(go, rng, threads)
    return y


def exact_adjoint(Y, p, threads=1):
    """x = scale * sum over rays (len * y) in FP64 (the exact transpose)."""
    L = lib()
    sd, sz, yd, zd, nz, dz = _exact_args(p)
    Y = _d(Y)
    nv, na, nb = len(sd), len(yd), len(zd)
    nvox = int(p["nx"]) * int(p["ny"]) * nz
    rng = _split(nv, threads)
    parts = [np.zeros(nvox, np.float64) for _ in rng]

    def go(k):
        a, b = rng[k]
        L.orc_exact_adjoint_f64(P(parts[k]), P(Y), D(float(p["SO"])), D(float(p["OD"])),
                                D(float(p["scale"])), I(int(p["nx"])), I(int(p["ny"])), I(nz),
                                D(dz), I(a), I(b), P(sd), P(sz), I(na), I(nb), P(yd), P(zd))
    if threads > 1 and len(rng) > 1:
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(go, range(len(rng))))
    else:
        for k in range(len(rng)):
            go(k)
    return np.sum(parts, axis=0)


def exact_count(p, views=None):
    """Voxels crossed with positive length, per ray (int64)."""
    L = lib()
    sd, sz, yd, zd, nz, dz = _exact_args(p)
    nv, na, nb = len(sd), len(yd), len(zd)
    v0, v1 = views or (0, nv)
    c = np.zeros((v1 - v0) * na * nb, np.int64)
    L.orc_exact_count(P(c), D(float(p["SO"])), D(float(p["OD"])), I(int(p["nx"])),
                      I(int(p["ny"])), I(nz), D(dz), I(v0), I(v1), P(sd), P(sz), I(na), I(nb),
                      P(yd), P(zd))
    return c


# --------------------------------------------------------------------------
# subsets: a list of rays or voxels at full problem size
# --------------------------------------------------------------------------
def _i64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64).reshape(-1))


def _chunks(n, threads):
    return _split(n, threads * 4 if threads > 1 else 1)


def exact_forward_rays(X, p, rays, threads=1):
    """FP64 exact forward of the rays ``rays`` (id iv*na*nb + ib*na + ia)."""
    L = lib()
    sd, sz, yd, zd, nz, dz = _exact_args(p)
    X = _d(X); rays = _i64(rays)
    y = np.zeros(rays.size, np.float64)

    def go(a, b):
        L.orc_exact_forward_rays(P(X), y[a:].ctypes.data_as(dp), D(float(p["SO"])),
                                 D(float(p["OD"])), D(float(p["scale"])), I(int(p["nx"])),
                                 I(int(p["ny"])), I(nz), D(dz), P(sd), P(sz), I(len(yd)),
                                 I(len(zd)), P(yd), P(zd), rays[a:].ctypes.data_as(i64p),
                                 C.c_long(b - a))
    _run(go, _chunks(rays.size, threads), threads)
    return y


def cone_siddon_rays(X, p, rays, threads=1):
    """Ax_cone_mf_cpu_siddon (Ax_cone_mf_cpu_siddon.cpp:19-134) for the rays
    ``rays``: each value is the one ``cone_siddon_f32`` writes, bit for bit."""
    L = lib()
    X = _f(X); sd = _f(p["sd_phi"]); sz = _f(p["sd_z"]); yd = _f(p["y_det"])
    zd = _f(p["z_det"]); idx = _i(p["id_X"]); rays = _i64(rays)
    y = np.zeros(rays.size, np.float32)

    def go(a, b):
        L.orc_cone_siddon_rays(P(X), y[a:].ctypes.data_as(fp), F(p["SO"]), F(p["OD"]),
                               F(p["scale"]), I(int(p["nx"])), I(int(p["ny"])), I(int(p["nz"])),
                               P(sd), P(sz), I(len(yd)), I(len(zd)), P(yd), P(zd), P(idx),
                               F(p["dz"]), rays[a:].ctypes.data_as(i64p), C.c_long(b - a))
    _run(go, _chunks(rays.size, threads), threads)
    return y


def exact_adjoint_vox(Y, p, vox, threads=1):
    """FP64 exact transpose of the FP32 sinogram ``Y`` at the voxels ``vox``
    (frame 0): the FP64 chord of every ray through each voxel, times the ray's
    value, summed in FP64."""
    L = lib()
    sd, sz, yd, zd, nz, dz = _exact_args(p)
    Y = _f(Y); vox = _i64(vox)
    x = np.zeros(vox.size, np.float64)

    def go(a, b):
        L.orc_exact_adjoint_vox(x[a:].ctypes.data_as(dp), P(Y), D(float(p["SO"])),
                                D(float(p["OD"])), D(float(p["scale"])), I(int(p["nx"])),
                                I(int(p["ny"])), I(nz), D(dz), I(0), I(len(sd)), P(sd), P(sz),
                                I(len(yd)), I(len(zd)), P(yd), P(zd),
                                vox[a:].ctypes.data_as(i64p), C.c_long(b - a))
    _run(go, _chunks(vox.size, threads), threads)
    return x


def cone_adj_vox(Y, p, vox, threads=1):
    """Atx_cone_mf_cpu_new (Atx_cone_mf_cpu_new.cpp:23-85) at the voxels ``vox``
    (frame 0): each value is the one ``cone_adj_f32`` writes, bit for bit."""
    L = lib()
    Y = _f(Y); cp = _f(p["cos_phi"]); sp = _f(p["sin_phi"]); sz = _f(p["sd_z"])
    yd = _f(p["y_det"]); zd = _f(p["z_det"]); idY = _i(np.asarray(p["id_Y"]).T.reshape(-1))
    Nv = _i(p["Nv"]); vox = _i64(vox)
    nx, ny, nz = int(p["nx"]), int(p["ny"]), int(p["nz"])
    x = np.zeros(vox.size, np.float32)

    def go(a, b):
        L.orc_cone_adj_vox(x[a:].ctypes.data_as(fp), P(Y), F(p["SO"]), F(p["OD"]),
                           F(p["scale"]), I(nx), I(ny), I(nz), P(sz), P(yd), P(zd),
                           F(p["dy_det"]), F(p["y_os"]), F(p["dz_det"]), F(p["dz"]), P(idY),
                           P(Nv), I(int(p["tmp_size"])), P(cp), P(sp), I(len(yd)), I(len(zd)),
                           vox[a:].ctypes.data_as(i64p), C.c_long(b - a))
    _run(go, _chunks(vox.size, threads), threads)
    return x


# --------------------------------------------------------------------------
# dominant-axis forward (version 1), FP32 restatement
# --------------------------------------------------------------------------
def cone_gao_f32(X, p, threads=1, views=None):
    """Ax_cone_mf_cpu_new (Ax_cone_mf_cpu_new.cpp:23-235): returns (y, yNorm)."""
    L = lib()
    X = _f(X); sd = _f(p["sd_phi"]); sz = _f(p["sd_z"]); yd = _f(p["y_det"])
    zd = _f(p["z_det"]); idx = _i(p["id_X"])
    nv, na, nb = len(sd), len(yd), len(zd)
    v0, v1 = views or (0, nv)
    y = np.zeros(nv * na * nb, np.float32)
    yn = np.zeros(nv * na * nb, np.float32)

    def go(a, b):
        L.orc_cone_gao_f32(P(X), P(y), P(yn), F(p["SO"]), F(p["OD"]), F(p["scale"]),
                           I(int(p["nx"])), I(int(p["ny"])), I(int(p["nz"])), I(a), I(b), P(sd),
                           P(sz), I(na), I(nb), P(yd), P(zd), P(idx), F(p["dz"]))
    rng = [(v0 + a, v0 + b) for a, b in _split(v1 - v0, threads * 4 if threads > 1 else 1)]
    _run(go, rng, threads)
    return y, yn


def fan_gao_f32(X, p, threads=1, views=None):
    """Ax_fan_mf_cpu_new (Ax_fan_mf_cpu_new.cpp:18-122)."""
    L = lib()
    X = _f(X); sd = _f(p["sd_phi"]); yd = _f(p["y_det"]); idx = _i(p["id_X"])
    nv, nd = len(sd), len(yd)
    v0, v1 = views or (0, nv)
    y = np.zeros(nv * nd, np.float32)

    def go(a, b):
        L.orc_fan_gao_f32(P(X), P(y), F(p["SO"]), F(p["OD"]), F(p["scale"]), I(int(p["nx"])),
                          I(int(p["ny"])), I(a), I(b), P(sd), I(nd), P(yd), P(idx))
    rng = [(v0 + a, v0 + b) for a, b in _split(v1 - v0, threads * 4 if threads > 1 else 1)]
    _run(go, rng, threads)
    return y


# --------------------------------------------------------------------------
# finite-size beam fan pair (version 2)
# --------------------------------------------------------------------------
def fan_fb_f32(X, p, threads=1):
    """Ax_fan_mf_cpu_new_fb (Ax_fan_mf_cpu_new_fb.cpp:19-123)."""
    L = lib()
    X = _f(X); sd = _f(p["sd_phi"]); yd = _f(p["y_det"]); idx = _i(p["id_X"])
    nv, nd = len(sd), len(yd)
    y = np.zeros(nv * nd, np.float32)

    def go(a, b):
        L.orc_fan_fb_f32(P(X), P(y), F(p["SO"]), F(p["OD"]), F(p["scale"]), I(int(p["nx"])),
                         I(int(p["ny"])), I(a), I(b), P(sd), I(nd), P(yd), P(idx),
                         F(p["dy_det"]))
    _run(go, _split(nv, threads * 4 if threads > 1 else 1), threads)
    return y


def fan_fb_adj_f32(Y, p, threads=1):
    """Atx_fan_mf_cpu_new_fb (Atx_fan_mf_cpu_new_fb.cpp:20-66), edges cos_det2/sin_det2."""
    L = lib()
    Y = _f(Y); cp = _f(p["cos_phi"]); sp = _f(p["sin_phi"]); cd = _f(p["cos_det2"])
    sdt = _f(p["sin_det2"]); idY = _i(np.asarray(p["id_Y"]).T.reshape(-1)); Nv = _i(p["Nv"])
    nx, ny, nt = int(p["nx"]), int(p["ny"]), int(p["nt"])
    nd = len(p["y_det"])
    x = np.zeros(nx * ny * nt, np.float32)

    def go(a, b):
        L.orc_fan_fb_adj_f32(P(x), P(Y), F(p["SO"]), F(p["OD"]), F(p["scale"]), I(nx), I(ny),
                             I(nd), F(p["dy_det"]), I(nt), P(idY), P(Nv), I(int(p["tmp_size"])),
                             P(cp), P(sp), P(cd), P(sdt), I(a), I(b))
    _run(go, _split(ny, threads * 4 if threads > 1 else 1), threads)
    return x


def ref_fan_fb(X, p):
    R = _need_ref()
    X = _f(X); sd = _f(p["sd_phi"]); yd = _f(p["y_det"]); idx = _i(p["id_X"])
    y = np.zeros(len(sd) * len(yd), np.float32)
    R.ref_Ax_fan_mf_cpu_new_fb(P(X), P(y), F(p["SO"]), F(p["OD"]), F(p["scale"]),
                               I(int(p["nx"])), I(int(p["ny"])), I(len(sd)), P(sd), I(len(yd)),
                               P(yd), P(idx), F(p["dy_det"]))
    return y


def ref_fan_fb_adj(Y, p):
    R = _need_ref()
    Y = _f(Y); sd = _f(p["sd_phi"]); yd = _f(p["y_det"]); cp = _f(p["cos_phi"])
    sp = _f(p["sin_phi"]); cd = _f(p["cos_det2"]); sdt = _f(p["sin_det2"])
    idY = _i(np.asarray(p["id_Y"]).T.reshape(-1)); Nv = _i(p["Nv"])
    nx, ny, nt = int(p["nx"]), int(p["ny"]), int(p["nt"])
    x = np.zeros(nx * ny * nt, np.float32)
    R.ref_Atx_fan_mf_cpu_new_fb(P(x), P(Y), F(p["SO"]), F(p["OD"]), F(p["scale"]), I(nx), I(ny),
                                P(sd), I(len(yd)), P(yd), F(p["dy_det"]), I(nt), P(idY), P(Nv),
                                I(int(p["tmp_size"])), I(int(p["nv"])), P(cp), P(sp), P(cd),
                                P(sdt))
    return x
