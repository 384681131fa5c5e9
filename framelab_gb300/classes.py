"""FrameLab's MATLAB class interface for the reconstruction path, over the
native library: the ``+DataTypes``, ``+Operators``, ``+Optimizers`` and
``+Transforms`` packages of ``matlab/classes``.

Names, argument order and meaning, and error messages follow the classes:
``ObjectData.m``, ``CTData.m``, ``FanBeamScanner.m``, ``ConeBeamScanner.m``,
``CGLS.m`` / ``solveCGLS.m``, ``SplitBregman.m`` / ``solveSplitBregman.m``,
``FrameletSystem.m`` and ``FrameletExpansion.m``. The projections and the
object algebra run on the GPU through the C ABI (``fl_forward``,
``fl_adjoint``, ``fl_axpby``, ``fl_dot``, ``fl_framelet_*``).

Arrays. A MATLAB array of size (Nx, Ny[, Nz]) is column-major. Here it is
held as a C-order float32 CUDA tensor of shape (Nz, Ny, Nx) / (Ny, Nx), which
has the same memory order. ``N`` and ``L`` are reported in MATLAB order
(x first). Sinograms are (nv, nb, na) for the cone beam and (nv, nd) for the
fan beam.

Models. By default a scanner uses the projector its ``para.version``
selects in the mex gateways, bit-exact with the reference's CPU kernels:
- fan forward: version 0 Siddon, 1 Gao, 2 finite beam;
- fan backprojection: versions 0 and 1 chord, 2 finite beam;
- cone forward: version 0 Siddon (``yNorm`` = 0, as the gateway leaves it),
  1 Gao with ``yNorm``;
- cone backprojection: chord.

``model='matched'`` selects the fast matched pair, whose backprojection is
the exact transpose of its forward.
"""
from __future__ import annotations

import ctypes as C
import math
from types import SimpleNamespace

import numpy as np
import torch

from . import _lib
from . import geometry as G
from .projector import Plan
from .transforms import FrameletSystem as _NativeFramelets



def _stream():
    return torch.cuda.current_stream().cuda_stream


def _dev(a) -> torch.Tensor:
    t = torch.as_tensor(a)
    return t.to(device="cuda", dtype=torch.float32).contiguous()


def _lin(a: float, x: torch.Tensor | None, b: float, y: torch.Tensor) -> torch.Tensor:
    """a*x + b*y as a new tensor (x None: b*y)."""
    z = y.clone()
    _lib.check(_lib.load().fl_axpby(z.data_ptr(), x.data_ptr() if x is not None else None,
                                    float(a), float(b), z.numel(), _stream()))
    return z


def _dot(x: torch.Tensor, y: torch.Tensor) -> float:
    out = torch.zeros(1, dtype=torch.float64, device=x.device)
    _lib.check(_lib.load().fl_dot(x.data_ptr(), y.data_ptr(), x.numel(), out.data_ptr(),
                                  _stream()))
    return float(out.item())


def _para_equal(p: dict, q: dict) -> bool:
    """structcmp: same fields, equal values."""
    if p.keys() != q.keys():
        return False
    return all(np.array_equal(np.asarray(p[k]), np.asarray(q[k])) for k in p)


# --------------------------------------------------------------------------
# +DataTypes
# --------------------------------------------------------------------------
class ObjectData:
    """ObjectData(dim, array, L) (ObjectData.m:13-51): an image / volume on a
    Cartesian grid of physical size L."""

    meshtype = "cartesian"

    def __init__(self, dim: int, array=None, L=None):
        if dim not in (2, 3):
            raise ValueError("dim must be 2 or 3")
        if array is None:
            array = torch.zeros((128,) * dim)
            L = (10.0,) * dim if L is None else L
        arr = _dev(array)
        if arr.dim() != dim:
            raise ValueError(f"array must have {dim} dimensions")
        self.dim = dim
        self.dataArray = arr
        self.N = tuple(int(s) for s in reversed(arr.shape))
        self.L = tuple(float(v) for v in (L if L is not None else (10.0,) * dim))
        self.Dx = tuple(l / n for l, n in zip(self.L, self.N))

    # algebra (ObjectData.m:84-116)
    def _check(self, b):
        if self.dim != b.dim or self.L != b.L:
            raise ValueError("Either dimensions or sizes are wrong!")

    def __add__(self, b):
        self._check(b)
        return ObjectData(self.dim, _lin(1.0, b.dataArray, 1.0, self.dataArray), self.L)

    def __sub__(self, b):
        self._check(b)
        return ObjectData(self.dim, _lin(-1.0, b.dataArray, 1.0, self.dataArray), self.L)

    def __neg__(self):
        return ObjectData(self.dim, _lin(0.0, None, -1.0, self.dataArray), self.L)

    def __rmul__(self, alpha):
        return ObjectData(self.dim, _lin(0.0, None, float(alpha), self.dataArray), self.L)

    __mul__ = __rmul__

    def objdot(self, b) -> float:
        """FP64 inner product of the data arrays (ObjectData.m:118-121)."""
        return _dot(self.dataArray, b.dataArray)

    def norm(self) -> float:
        return math.sqrt(self.objdot(self))

    def frameletTransform(self, sys):
        return sys.forwardTransform(self.dataArray)

    def adjointFrameletTransform(self, sys, alpha):
        self.dataArray = alpha.adjointFrameletTransform(sys)

    def applyOperator(self, oper):
        return oper.apply(self)

    def updateDataArray(self, A):
        self.dataArray = _dev(A)


class CTData:
    """CTData(scanner, dataArray, dataArrayNorm, L) (CTData.m:16-24): projection
    data of a scanner, with the normalised projections of the cone forward."""

    def __init__(self, scanner, dataArray, dataArrayNorm, L):
        self.scanner = scanner
        self.dataArray = _dev(dataArray)
        self.dataArrayNorm = None if dataArrayNorm is None else _dev(dataArrayNorm)
        self.L = tuple(L)

    @property
    def para(self):
        return self.scanner.para

    def _norm_lin(self, a, b, bn):
        if self.dataArrayNorm is None or bn is None:
            return None
        return _lin(a, bn, 1.0, self.dataArrayNorm)

    def __add__(self, b):
        if isinstance(b, CTData):
            if tuple(self.dataArray.shape) != tuple(b.dataArray.shape):
                raise ValueError("Array dimension mismatch!")
            return CTData(self.scanner, _lin(1.0, b.dataArray, 1.0, self.dataArray),
                          self._norm_lin(1.0, b, b.dataArrayNorm), self.L)
        n = None if self.dataArrayNorm is None else self.dataArrayNorm + b
        return CTData(self.scanner, self.dataArray + b, n, self.L)

    def __sub__(self, b):
        if tuple(self.dataArray.shape) != tuple(b.dataArray.shape):
            raise ValueError("Array dimension mismatch!")
        return CTData(self.scanner, _lin(-1.0, b.dataArray, 1.0, self.dataArray),
                      self._norm_lin(-1.0, b, b.dataArrayNorm), self.L)

    def __neg__(self):
        n = None if self.dataArrayNorm is None else _lin(0.0, None, -1.0, self.dataArrayNorm)
        return CTData(self.scanner, _lin(0.0, None, -1.0, self.dataArray), n, self.L)

    def __rmul__(self, alpha):
        n = (None if self.dataArrayNorm is None
             else _lin(0.0, None, float(alpha), self.dataArrayNorm))
        return CTData(self.scanner, _lin(0.0, None, float(alpha), self.dataArray), n, self.L)

    __mul__ = __rmul__

    def objdot(self, b) -> float:
        return _dot(self.dataArray, b.dataArray)

    def frameletTransform(self, sys):
        return sys.forwardTransform(self.dataArray)


class FrameletExpansion:
    """FrameletExpansion(dim, frameletSystem, frameletArray): the coefficient
    set of a FrameletSystem, held as one flat device array (all levels and
    bands; the layout of ``transforms.FrameletSystem``)."""

    def __init__(self, dim: int, frameletSystem, frameletArray: torch.Tensor):
        self.dim = dim
        self.frameletSystem = frameletSystem
        self.frameletArray = frameletArray

    def _like(self, arr):
        return FrameletExpansion(self.dim, self.frameletSystem, arr)

    def _check(self, b):
        if self.dim != b.dim:
            raise ValueError(f"warning: inconsistent dimensions: a.dim = {self.dim}b.dim = {b.dim}")

    def __add__(self, b):
        self._check(b)
        return self._like(_lin(1.0, b.frameletArray, 1.0, self.frameletArray))

    def __sub__(self, b):
        self._check(b)
        return self._like(_lin(-1.0, b.frameletArray, 1.0, self.frameletArray))

    def __rmul__(self, alpha):
        return self._like(_lin(0.0, None, float(alpha), self.frameletArray))

    __mul__ = __rmul__

    def softThreshold(self, tau: float):
        """In place: sign(a) max(|a| - tau, 0) on every band except the low band
        of the coarsest level (softThreshold.m:47-80)."""
        nat = self.frameletSystem._native
        _lib.check(_lib.load().fl_framelet_shrink(nat._h, self.frameletArray.data_ptr(),
                                                  self.frameletArray.data_ptr(), float(tau),
                                                  _stream()))

    def adjointFrameletTransform(self, sys=None) -> torch.Tensor:
        return (sys or self.frameletSystem).adjointTransform(self)


# --------------------------------------------------------------------------
# +Transforms
# --------------------------------------------------------------------------
class FrameletSystem:
    """FrameletSystem(dim, type, level) (FrameletSystem.m:12-64): undecimated
    B-spline framelets ('haar', 'linear', 'cubic'), circular boundary. The
    native transform is built for the array shape at first use."""

    def __init__(self, dim: int = 2, type: str = "haar", level: int = 1):
        if type not in ("haar", "linear", "cubic"):
            raise ValueError("type must be 'haar', 'linear' or 'cubic'")
        self.dim, self.type, self.level = dim, type, level
        self._native = None

    def _for(self, shape):
        shape = tuple(int(s) for s in shape)
        if len(shape) != self.dim:
            raise ValueError(f"array must have {self.dim} dimensions")
        if self._native is None or self._native.shape != shape:
            self._native = _NativeFramelets(shape, self.type, self.level)
        return self._native

    def forwardTransform(self, u) -> FrameletExpansion:
        if isinstance(u, ObjectData):
            u = u.dataArray
        u = _dev(u)
        return FrameletExpansion(self.dim, self, self._for(u.shape).forward(u))

    def adjointTransform(self, alpha) -> torch.Tensor:
        coef = alpha.frameletArray if isinstance(alpha, FrameletExpansion) else alpha
        if self._native is None:
            raise ValueError("adjointTransform before any forwardTransform: shape unknown")
        return self._native.adjoint(coef)


# --------------------------------------------------------------------------
# +Operators
# --------------------------------------------------------------------------
class _Scanner:
    """Plans are built once per object geometry and reused (the reference
    rebuilds its ``para`` struct at every ``apply``; the values are the same)."""

    def _plan(self, key, make_para) -> Plan:
        plans = self.__dict__.setdefault("_plans", {})
        if key not in plans:
            para = make_para()
            plans[key] = (para, Plan(para))
        return plans[key]


class FanBeamScanner(_Scanner):
    """FanBeamScanner(nd, nv) (FanBeamScanner.m): flat-detector fan beam with
    the class defaults SO = OD = 5, Ly = 6 (in the object's length unit)."""

    scanType = "2DFan"

    def __init__(self, nd: int = 256, nv: int = 256, SO=5.0, OD=5.0, Ly=6.0, y_os=0.0,
                 version: int = 1, model: str | None = None):
        self.nd, self.nv = int(nd), int(nv)
        self.SO, self.OD, self.Ly, self.y_os = float(SO), float(OD), float(Ly), float(y_os)
        self.version, self.model = int(version), model
        self.para = {}
        self.verbose = False

    def _make_para(self, N, L):
        """FanBeamScanner/setPara.m:1-57 for an object of size N, L."""
        nx, ny = N
        return G.fan_para(nx, ny, self.nd, self.nv, L=L, SO=self.SO, OD=self.OD, Ly=self.Ly,
                          y_os=self.y_os, version=self.version)

    def setPara(self, obj: ObjectData):
        key = ("object", obj.N, obj.L)
        self.para, self._P = self._plan(key, lambda: self._make_para(obj.N, obj.L))

    def apply(self, obj: ObjectData) -> CTData:
        self.setPara(obj)
        model = self.model or {0: "siddon_ref", 1: "gao_ref", 2: "fb_ref"}[self.version]
        y = self._P.forward(obj.dataArray.reshape(-1), model=model)
        return CTData(self, y.reshape(self.nv, self.nd), None, obj.L)

    def applyAdjoint(self, data: CTData) -> ObjectData:
        if not self.para:
            self.para, self._P = data.scanner.para, data.scanner._P
        elif not _para_equal(self.para, data.scanner.para):
            raise ValueError("Object scan parameters and scanner parameters do not agree!")
        model = self.model or ("fb_ref" if self.version == 2 else "chord_ref")
        x = self._P.adjoint(data.dataArray.reshape(-1), model=model)
        return ObjectData(2, x.reshape(int(self.para["ny"]), int(self.para["nx"])), data.L)


class ConeBeamScanner(_Scanner):
    """ConeBeamScanner(type, na, nb, nv, zmax, rps, vtab, fps, nHelix, phaseShift)
    (ConeBeamScanner.m:35-78): 'circle', 'helix' or 'multiHelix' scans with
    the class defaults SO = OD = 5, Ly = Lz = 6."""

    def __init__(self, type=None, na=None, nb=None, nv=None, zmax=None, rps=3.0, vtab=2.0,
                 fps=30.0, nHelix=1, phaseShift=0.0, SO=5.0, OD=5.0, Ly=6.0, Lz=6.0,
                 version: int = 1, model: str | None = None):
        if type is None or na is None or nb is None or (nv is None and zmax is None):
            raise ValueError("You must specify type, na, nb and nv")
        if type not in ("circle", "helix", "multiHelix"):
            raise ValueError("circle, helix and multiHelix are only valid types")
        if type == "circle" and zmax is not None:
            raise ValueError("zmax, rps, vtab, fps are for helical scan only")
        if type != "circle" and zmax is None:
            raise ValueError("helix and multiHelix require more inputs")
        self.type, self.na, self.nb = type, int(na), int(nb)
        self.zmax, self.rps, self.vtab, self.fps = zmax, float(rps), float(vtab), float(fps)
        self.nHelix = int(nHelix)
        self.phaseShift = np.atleast_1d(np.asarray(phaseShift, dtype=np.float64))
        if type == "circle":
            self.nv = int(nv)
        else:
            per = int(math.floor(self.fps * float(zmax) / self.vtab)) + 1
            self.nv = per * (self.nHelix if type == "multiHelix" else 1)
        self.SO, self.OD, self.Ly, self.Lz = float(SO), float(OD), float(Ly), float(Lz)
        self.version, self.model = int(version), model
        self.para = {}
        self.verbose = False
        self.GPU = 1

    def _make_para(self, N, L):
        """ConeBeamScanner/setPara.m:1-84 for an object of size N, L."""
        nx, ny, nz = N
        kw = {}
        if self.type != "circle":
            kw = dict(zmax=float(self.zmax), rps=self.rps, vtab=self.vtab, fps=self.fps,
                      n_helix=self.nHelix, phase_shift=tuple(self.phaseShift))
        return G.cone_para(nx, ny, nz, self.na, self.nb, self.nv, L=L, SO=self.SO, OD=self.OD,
                           Ly=self.Ly, Lz=self.Lz, scan=self.type, version=self.version, **kw)

    def setPara(self, obj: ObjectData):
        key = ("object", obj.N, obj.L)
        self.para, self._P = self._plan(key, lambda: self._make_para(obj.N, obj.L))

    def _shape(self, t: torch.Tensor) -> torch.Tensor:
        if self.type == "multiHelix":
            return t.reshape(self.nHelix, self.nv // self.nHelix, self.nb, self.na)
        return t.reshape(self.nv, self.nb, self.na)

    def apply(self, obj: ObjectData) -> CTData:
        self.setPara(obj)
        P = self._P
        x = obj.dataArray.reshape(-1)
        model = self.model or ("siddon_ref" if self.version == 0 else "gao_ref")
        if model == "gao_ref":
            y, yn = P.forward_gao(x, with_norm=True)
        else:
            y = P.forward(x, model=model)
            yn = torch.zeros_like(y)
        return CTData(self, self._shape(y), self._shape(yn), obj.L)

    def applyAdjoint(self, data: CTData, N) -> ObjectData:
        """Backprojection onto an N = [nx, ny, nz] grid with the voxel size of
        the projected object (applyAdjoint.m:1-41)."""
        if not self.para:
            self.para = data.scanner.para
        elif not _para_equal(self.para, data.scanner.para):
            raise ValueError("Object scan parameters and scanner parameters do not agree!")
        nx, ny, nz = (int(v) for v in N)
        base = self.para

        def make():
            para = dict(base)
            para.update(nx=np.uint32(nx), ny=np.uint32(ny), nz=np.uint32(nz))
            return para
        _, P = self._plan(("adjoint", id(base), (nx, ny, nz)), make)
        model = self.model or "chord_ref"
        x = P.adjoint(data.dataArray.reshape(-1), model=model)
        return ObjectData(3, x.reshape(nz, ny, nx), data.L)


# --------------------------------------------------------------------------
# +Optimizers
# --------------------------------------------------------------------------
class CGLS:
    """CGLS(A, At, b, u0, lam, globalIter, convergenceTol) (CGLS.m:21-44):
    (At A + lam I) u = b for operators on objects with objdot, + and scalar *."""

    def __init__(self, A=None, At=None, b=None, u0=None, lam=None, globalIter=500,
                 convergenceTol=1e-14):
        if A is None or At is None or b is None or u0 is None or lam is None:
            raise ValueError("CGLS requires A, At, b, u0 and lam")
        self.A, self.At, self.b, self.u0, self.lam = A, At, b, u0, float(lam)
        self.globalIter, self.convergenceTol = int(globalIter), float(convergenceTol)
        self.history = []

    def solveCGLS(self):
        """solveCGLS.m:6-31."""
        lam = self.lam
        A_loc = lambda x: self.At(self.A(x)) + lam * x  # noqa: E731
        rk = A_loc(self.u0) - self.b
        pk = -rk
        uk = self.u0
        gammaold = rk.objdot(rk)
        self.history = []
        icg = 0
        while icg < self.globalIter:
            icg += 1
            qk = A_loc(pk)
            alphak = gammaold / pk.objdot(qk)
            uk = uk + alphak * pk
            rk = rk + alphak * qk
            gammanew = rk.objdot(rk)
            self.history.append(gammanew)
            betak = gammanew / gammaold
            pk = -rk + betak * pk
            gammaold = gammanew
            if gammaold < self.convergenceTol:
                icg = self.globalIter
        return uk


class SplitBregman:
    """SplitBregman(A, At, W, Wt, lam, mu, f, u0, globalIter, cgIter, cgTol)
    (SplitBregman.m:20-43): min 1/2 |A u - f|^2 + lam |W u|_1."""

    def __init__(self, A=None, At=None, W=None, Wt=None, lam=None, mu=None, f=None, u0=None,
                 globalIter=1, cgIter=10, cgTol=1e-10):
        if any(v is None for v in (A, At, W, Wt, lam, f, u0)):
            raise ValueError("SplitBregman requires A,At,W,Wt,lam,f,and u0")
        self.A, self.At, self.W, self.Wt = A, At, W, Wt
        self.lam, self.mu = float(lam), float(mu)
        self.f, self.u0 = f, u0
        self.globalIter, self.cgIter, self.cgTol = int(globalIter), int(cgIter), float(cgTol)

    def solveSplitBregman(self):
        """solveSplitBregman.m:1-41 (Lagrange update v = v + (Wu - alpha))."""
        A, At, W, Wt, mu = self.A, self.At, self.W, self.Wt, self.mu
        alpha = W(self.u0)
        v = alpha
        Atf = At(self.f)
        b = Atf + mu * Wt(alpha - v)
        cg = CGLS(A, At, b, self.u0, mu, self.cgIter, self.cgTol)
        u = self.u0
        for _ in range(self.globalIter):
            u = cg.solveCGLS()
            Wu = W(u)
            alpha = v + Wu
            alpha.softThreshold(self.lam / mu)
            v = v + (Wu - alpha)
            b = Atf + mu * Wt(alpha - v)
            cg = CGLS(A, At, b, u, mu, self.cgIter, self.cgTol)
        return u


DataTypes = SimpleNamespace(ObjectData=ObjectData, CTData=CTData,
                            FrameletExpansion=FrameletExpansion)
Operators = SimpleNamespace(FanBeamScanner=FanBeamScanner, ConeBeamScanner=ConeBeamScanner)
Optimizers = SimpleNamespace(CGLS=CGLS, SplitBregman=SplitBregman)
Transforms = SimpleNamespace(FrameletSystem=FrameletSystem)
