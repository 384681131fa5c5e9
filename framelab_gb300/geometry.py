"""Scanner geometry -> the ``para`` parameter struct of FrameLab's mex kernels.

Mirrors ``FanBeamScanner/setPara.m:1-57`` and ``ConeBeamScanner/setPara.m:1-84``:
everything is rescaled so the xy voxel pitch is 1 (``scale = Dx(1)``), the
detector grids are pixel-centred, and the frame bookkeeping (``id_X``, ``id_Y``,
``Nv``, ``tmp_size``) describes a single frame (``nt = 1``), as the reference's
classes always do.

Arithmetic follows MATLAB's class rules operation by operation:
* both operands ``single`` (the scanner's ``SO``, ``OD``, ``Ly``, ``Lz`` and
  ``y_os`` properties, ``ConeBeamScanner.m:10-16``, ``FanBeamScanner.m:5-10``,
  and ``scale``): the operation is a single-precision one;
* one operand ``double`` (the counts ``na``, ``nb``, ``nd``, the helix step
  ``h``, index ranges): the operation is carried out in double and its result
  rounded to ``single``;
* an all-``double`` expression wrapped in ``single(...)`` is rounded once.
Each field below cites the ``setPara.m`` line whose order it follows.
MATLAB's own single-precision ``cos``/``sin``/``atan2`` are not available
here; they are taken as the double-precision result rounded to single.

Field names and dtypes are those the mex gateways read (``Ax_fan_mf.cpp:28-41``,
``Atx_fan_mf.cpp:29-63``, ``Ax_cone_mf.cpp:31-52``, ``Atx_cone_mf.cpp:31-55``) and
``checkInputs.m`` enforces (``single`` and ``uint32``).
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32
u32 = np.uint32


def _single_trig(fn, x):
    return fn(np.asarray(x, dtype=np.float64)).astype(np.float32)


def _mixed(a_double, b_single) -> np.ndarray:
    """One MATLAB operation ``double * single``: computed in double, rounded
    to single."""
    return (np.asarray(a_double, np.float64) * np.float64(b_single)).astype(np.float32) \
        if np.ndim(b_single) == 0 else \
        (np.float64(a_double) * np.asarray(b_single, np.float32).astype(np.float64)).astype(
            np.float32)


def _pitch(L_single, n: int) -> np.float32:
    """``L/n`` with ``L`` a single property and ``n`` a double count
    (``FanBeamScanner/setPara.m:10``, ``ConeBeamScanner/setPara.m:10-11``):
    the division runs in double and rounds to single."""
    return f32(np.float64(f32(L_single)) / np.float64(n))


def _centred_grid(n: int, pitch: np.float32, offset: np.float32) -> np.ndarray:
    """``single(((-n/2:n/2-1)+0.5)*pitch + offset)``
    (``FanBeamScanner/setPara.m:23``, ``ConeBeamScanner/setPara.m:53-54``):
    the double index vector times the single pitch is one mixed operation
    (double product, exact here, rounded to single), then a single + single
    addition of the offset."""
    k = -n / 2.0 + np.arange(n, dtype=np.float64) + 0.5
    return (_mixed(k, f32(pitch)) + f32(offset)).astype(np.float32)


def _frame_tables(nv: int):
    """Single-frame bookkeeping of setPara.m (FanBeamScanner/setPara.m:33-52)."""
    id_X = np.zeros(nv, dtype=np.uint32)
    id_Y = np.arange(nv, dtype=np.uint32).reshape(nv, 1)
    Nv = np.array([nv], dtype=np.uint32)
    return id_X, id_Y, Nv, u32(nv)


def fan_para(nx: int, ny: int, nd: int, nv: int, L=(10.0, 10.0), SO=5.0, OD=5.0,
             Ly=6.0, y_os=0.0, sd_phi=None, version=1) -> dict:
    """``para`` for a fan-beam scan of an ``nx x ny`` image of physical size ``L``.

    Defaults are the reference's ``FanBeamScanner`` properties (SO = OD = 5,
    Ly = 6, ``FanBeamScanner.m:4-11``); ``sd_phi`` overrides the uniform 2*pi
    source angles.
    """
    scale = f32(L[0] / nx)                          # single(object.Dx(1))  (setPara.m:5)
    SOs, ODs = f32(SO) / scale, f32(OD) / scale     # single / single       (setPara.m:8-9)
    dy_det = _pitch(Ly, nd)                         # Ly / nd               (setPara.m:10)
    if sd_phi is None:
        sd_phi = (2 * math.pi / nv * np.arange(nv)).astype(np.float32)
    sd_phi = np.asarray(sd_phi, dtype=np.float32)
    y_det = (_centred_grid(nd, dy_det, f32(y_os)) / scale).astype(np.float32)
    angle_det = np.arctan2(y_det.astype(np.float64),
                           np.float64(f32(SOs + ODs))).astype(np.float32)
    id_X, id_Y, Nv, tmp = _frame_tables(len(sd_phi))
    # bin edges for the finite-beam model (version 2): cos_det2/sin_det2, nd + 1
    # entries, read by Atx_fan_mf.cpp:38-44
    k = (-nd / 2.0 + np.arange(nd + 1, dtype=np.float64)).astype(np.float32)
    edges = ((k * dy_det + f32(y_os)) / scale).astype(np.float32)
    angle_edge = np.arctan2(edges.astype(np.float64),
                            np.float64(f32(SOs + ODs))).astype(np.float32)
    return dict(
        SO=f32(SOs), OD=f32(ODs), dy_det=f32(dy_det / scale), y_os=f32(0.0),
        cos_det2=_single_trig(np.cos, angle_edge), sin_det2=_single_trig(np.sin, angle_edge),
        scale=scale, nx=u32(nx), ny=u32(ny), nt=u32(1), sd_phi=sd_phi, y_det=y_det,
        cos_phi=_single_trig(np.cos, sd_phi), sin_phi=_single_trig(np.sin, sd_phi),
        cos_det=_single_trig(np.cos, angle_det), sin_det=_single_trig(np.sin, angle_det),
        id_X=id_X, id_Y=id_Y, Nv=Nv, nv=u32(len(sd_phi)), tmp_size=tmp,
        version=u32(version), GPU=u32(1),
    )


def fan_para_equiangular(nx: int, ny: int, nd: int, nv: int, L, SO, SD, fan_angle,
                         version=1) -> dict:
    """Fan-beam ``para`` for an equiangular (arc) detector of ``nd`` bins that
    together span ``fan_angle`` radians.

    The reference supports only a flat panel (``Ax_fan_mf_cpu_siddon.cpp:38-39``).
    A ray is fixed by its source and one point on it, so an arc bin at angle
    gamma is expressed as the flat-panel point ``SD*tan(gamma)`` on the panel
    at distance OD from the isocentre; the projector sees the same rays.
    """
    p = fan_para(nx, ny, nd, nv, L=L, SO=SO, OD=SD - SO, Ly=1.0, version=version)
    SDs = np.float64(p["SO"]) + np.float64(p["OD"])
    dgam = fan_angle / nd
    gam = (np.arange(nd) - nd / 2 + 0.5) * dgam
    y_det = (SDs * np.tan(gam)).astype(np.float32)
    angle_det = np.arctan2(y_det.astype(np.float64), SDs).astype(np.float32)
    p.update(y_det=y_det, cos_det=_single_trig(np.cos, angle_det),
             sin_det=_single_trig(np.sin, angle_det),
             dy_det=f32(SDs * dgam), det_arc=True, det_gamma0=float(gam[0]),
             det_dgamma=float(dgam))
    return p


def cone_para(nx: int, ny: int, nz: int, na: int, nb: int, nv: int = 128,
              L=(10.0, 10.0, 10.0), SO=5.0, OD=5.0, Ly=6.0, Lz=6.0, y_os=0.0,
              scan="circle", zmax=2.0, rps=3.0, vtab=2.0, fps=30.0, n_helix=1,
              phase_shift=(0.0,), nv_block=4, version=1) -> dict:
    """``para`` for a cone-beam scan (``ConeBeamScanner/setPara.m:1-84``).

    ``scan`` is ``'circle'``, ``'helix'`` or ``'multiHelix'``; for the helical
    scans the view count follows ``ConeBeamScanner.m:53-58``.
    """
    scale = f32(L[0] / nx)                          # single(object.Dx(1))      (setPara.m:5)
    dzv = f32(f32(L[2] / nz) / scale)               # single(object.Dx(3))/scale (setPara.m:22)
    SOs, ODs = f32(SO) / scale, f32(OD) / scale     # single / single           (setPara.m:8-9)
    dy_det = _pitch(Ly, na)                         # Ly / na                   (setPara.m:10)
    dz_det = _pitch(Lz, nb)                         # Lz / nb                   (setPara.m:11)
    pdy, pdz = f32(dy_det / scale), f32(dz_det / scale)   # single / single   (setPara.m:12-13)
    if scan == "circle":
        sd_phi = (2 * math.pi / nv * np.arange(nv)).astype(np.float32)
        sd_z = (np.zeros(nv, dtype=np.float32) / scale).astype(np.float32)
    elif scan in ("helix", "multiHelix"):
        phi_max = rps * zmax * 2 * math.pi / vtab
        dphi = 2 * math.pi * rps / fps
        nper = int(math.floor(phi_max / dphi + 1e-10)) + 1
        base = -phi_max / 2 + dphi * np.arange(nper)
        h = vtab / (2 * math.pi * rps)
        shifts = [0.0] if scan == "helix" else list(phase_shift)[:n_helix]
        # single((-phiMax/2:dphi:phiMax/2) + phaseShift(i))  (setPara.m:32, 42)
        phis = [(base + s).astype(np.float32) for s in shifts]
        sd_phi = np.concatenate(phis).astype(np.float32)
        if scan == "helix":
            # single(h*sd_phi)/scale: double h times the single sd_phi is a
            # mixed operation (double product rounded to single)  (setPara.m:35)
            zs = [(_mixed(h, sd_phi) / scale).astype(np.float32)]
        else:
            # single(h*(-phiMax/2:dphi:phiMax/2))/scale: all double, rounded
            # once, the same z for every helix  (setPara.m:49)
            zs = [((h * base).astype(np.float32) / scale).astype(np.float32) for _ in shifts]
        sd_z = np.concatenate(zs).astype(np.float32)
    else:
        raise ValueError("circle, helix and multiHelix are only valid types")
    nvv = len(sd_phi)
    y_det = (_centred_grid(na, dy_det, f32(y_os)) / scale).astype(np.float32)
    z_det = (_centred_grid(nb, dz_det, f32(0.0)) / scale).astype(np.float32)
    id_X, id_Y, Nv, tmp = _frame_tables(nvv)
    return dict(
        SO=f32(SOs), OD=f32(ODs), dy_det=pdy, dz_det=pdz, y_os=f32(f32(y_os) / pdy),
        scale=scale, nx=u32(nx), ny=u32(ny), nz=u32(nz), dz=dzv, nt=u32(1),
        sd_phi=sd_phi, sd_z=sd_z, y_det=y_det, z_det=z_det,
        cos_phi=_single_trig(np.cos, sd_phi), sin_phi=_single_trig(np.sin, sd_phi),
        id_X=id_X, id_Y=id_Y, Nv=Nv, nv=u32(nvv), tmp_size=tmp,
        nv_block=u32(nv_block), version=u32(version), GPU=u32(1),
    )


def cone_para_mm(n: int, nv: int, na: int, nb: int, det_pitch_mm: float, SO_mm: float,
                 SD_mm: float, voxel_mm: float, nz: int | None = None, **kw) -> dict:
    """Cone ``para`` from scanner units: an ``n x n x nz`` volume of ``voxel_mm``
    voxels, a ``na x nb`` flat panel of ``det_pitch_mm`` pixels, source-isocentre
    ``SO_mm`` and source-detector ``SD_mm`` distances."""
    nz = n if nz is None else nz
    L = (n * voxel_mm, n * voxel_mm, nz * voxel_mm)
    return cone_para(n, n, nz, na, nb, nv, L=L, SO=SO_mm, OD=SD_mm - SO_mm,
                     Ly=na * det_pitch_mm, Lz=nb * det_pitch_mm, **kw)
