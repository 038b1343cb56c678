"""Optical components and material models with ROBAST's API.

Mirrors the reference classes
  AOpticalComponent / AMirror / ALens / AFocalSurface / AObscuration
      (include/AOpticalComponent.h:22-41, include/AMirror.h:24-46,
       include/ALens.h:23-40, include/AFocalSurface.h:22-39,
       include/AObscuration.h:20-29)
  ABorderSurfaceCondition            (include/ABorderSurfaceCondition.h:24-48)
  ARefractiveIndex / ASellmeierFormula / ACauchyFormula / ASchottFormula /
  AMixedRefractiveIndex / AFilmetrixDotCom / AGlassCatalog
  AMultilayer                         (include/AMultilayer.h)
and the ROOT helpers TGraph / TGraph2D / TH2 used as lookup tables.
Objects only record parameters; evaluation happens in the native library.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from typing import List, Optional

import numpy as np

from . import _native as N
from .geometry import TGeoBBox, TGeoMatrix, TGeoShape


# ---------------------------------------------------------------------------
# lookup tables
# ---------------------------------------------------------------------------
class TGraph:
    """Piecewise-linear table with TGraph::Eval semantics."""

    def __init__(self, n: int = 0, x=None, y=None):
        self.x: List[float] = []
        self.y: List[float] = []
        if x is not None:
            self.x = [float(v) for v in x]
            self.y = [float(v) for v in y]

    def SetPoint(self, i, x, y):
        while len(self.x) <= i:
            self.x.append(0.0)
            self.y.append(0.0)
        self.x[i], self.y[i] = float(x), float(y)

    def GetN(self):
        return len(self.x)

    def Eval(self, x):
        """TGraph::Eval: linear interpolation between the neighbours of x,
        linear extrapolation with the end pairs, exact match returns y."""
        xs = np.asarray(self.x)
        ys = np.asarray(self.y)
        order = np.argsort(xs, kind="stable")
        xs, ys = xs[order], ys[order]
        n = len(xs)
        if n == 1:
            return float(ys[0])
        hit = np.nonzero(xs == x)[0]
        if len(hit):
            return float(ys[hit[0]])
        if x < xs[0]:
            lo, hi = 0, 1
        elif x > xs[-1]:
            lo, hi = n - 2, n - 1
        else:
            hi = 1
            while hi < n - 1 and xs[hi] < x:
                hi += 1
            lo = hi - 1
        if xs[hi] == xs[lo]:
            return float(ys[lo])
        return float(ys[lo] + (x - xs[lo]) * (ys[hi] - ys[lo]) / (xs[hi] - xs[lo]))


class TGraph2D:
    """2D table.  Points must form a complete rectilinear grid; it is
    interpolated bilinearly (for such grids this agrees with TGraph2D's
    Delaunay interpolation on the cell diagonals and at the nodes)."""

    def __init__(self):
        self.pts = []

    def SetPoint(self, i, x, y, z):
        while len(self.pts) <= i:
            self.pts.append((0.0, 0.0, 0.0))
        self.pts[i] = (float(x), float(y), float(z))

    def grid(self):
        xs = sorted({p[0] for p in self.pts})
        ys = sorted({p[1] for p in self.pts})
        z = np.full((len(xs), len(ys)), np.nan)
        for x, y, v in self.pts:
            z[xs.index(x), ys.index(y)] = v
        if np.isnan(z).any():
            raise ValueError("TGraph2D points do not form a rectilinear grid")
        return np.array(xs), np.array(ys), z

    def Interpolate(self, x, y):
        xs, ys, z = self.grid()
        return _bilinear(xs, ys, z, x, y)


class TH2:
    """Histogram-backed table (TH2::Interpolate on bin centres)."""

    def __init__(self, xcenters, ycenters, values):
        self.xs = np.asarray(xcenters, dtype=float)
        self.ys = np.asarray(ycenters, dtype=float)
        self.z = np.asarray(values, dtype=float).reshape(len(self.xs), len(self.ys))

    def grid(self):
        return self.xs, self.ys, self.z

    def Interpolate(self, x, y):
        return _bilinear(self.xs, self.ys, self.z, x, y)


def _bilinear(xs, ys, z, x, y):
    def frac(a, v):
        if len(a) == 1:
            return 0, 0.0
        if v <= a[0]:
            return 0, 0.0
        if v >= a[-1]:
            return len(a) - 2, 1.0
        i = int(np.searchsorted(a, v, side="right") - 1)
        i = min(max(i, 0), len(a) - 2)
        return i, (v - a[i]) / (a[i + 1] - a[i])

    ix, fx = frac(xs, x)
    iy, fy = frac(ys, y)
    ix1 = ix + 1 if len(xs) > 1 else ix
    iy1 = iy + 1 if len(ys) > 1 else iy
    return float((1 - fx) * (1 - fy) * z[ix, iy] + (1 - fx) * fy * z[ix, iy1] + fx * (1 - fy) * z[ix1, iy]
                 + fx * fy * z[ix1, iy1])


# ---------------------------------------------------------------------------
# refractive indices
# ---------------------------------------------------------------------------
class ARefractiveIndex:
    """n(lambda), k(lambda) from TGraphs; ARefractiveIndex(n, k) is a
    constant (include/ARefractiveIndex.h:25-68, src/ARefractiveIndex.cxx)."""

    kind = N.INDEX_TABLE

    def __init__(self, n: Optional[float] = None, k: float = 0.0):
        self.n_graph: Optional[TGraph] = None
        self.k_graph: Optional[TGraph] = None
        if n is not None:
            self.n_graph = TGraph()
            self.n_graph.SetPoint(0, 0.0, n)
            if k > 0:
                self.k_graph = TGraph()
                self.k_graph.SetPoint(0, 0.0, k)

    def SetRefractiveIndex(self, g: TGraph):
        self.n_graph = g

    def SetExtinctionCoefficient(self, g: TGraph):
        self.k_graph = g

    def coefficients(self):
        return [0.0] * 6

    def GetRefractiveIndex(self, lam):
        return self.n_graph.Eval(lam) if self.n_graph is not None else 1.0

    def GetExtinctionCoefficient(self, lam):
        return self.k_graph.Eval(lam) if self.k_graph is not None else 0.0

    def GetAbsorptionLength(self, lam):
        k = self.GetExtinctionCoefficient(lam)
        return math.inf if k <= 0 else self.ExtinctionCoefficientToAbsorptionLength(k, lam)

    def GetComplexRefractiveIndex(self, lam):
        return complex(self.GetRefractiveIndex(lam), self.GetExtinctionCoefficient(lam))

    def GetAbbeNumber(self):
        nm = 1e-7
        nC = self.GetRefractiveIndex(656.2725 * nm)
        nD = self.GetRefractiveIndex(589.2938 * nm)
        nF = self.GetRefractiveIndex(486.1327 * nm)
        return (nD - 1.0) / (nF - nC)

    @staticmethod
    def AbsorptionLengthToExtinctionCoefficient(a, lam):
        return lam / (4 * math.pi * a)

    @staticmethod
    def ExtinctionCoefficientToAbsorptionLength(k, lam):
        return lam / (4 * math.pi * k)


class ASellmeierFormula(ARefractiveIndex):
    """n^2 = 1 + sum B_i l^2 / (l^2 - C_i), l in um (src/ASellmeierFormula.cxx:46-54)."""

    kind = N.INDEX_SELLMEIER

    def __init__(self, B1, B2, B3, C1, C2, C3):
        super().__init__()
        self.par = [float(v) for v in (B1, B2, B3, C1, C2, C3)]

    def coefficients(self):
        return list(self.par)

    def GetRefractiveIndex(self, lam):
        l2 = (lam / 1e-4) ** 2
        B1, B2, B3, C1, C2, C3 = self.par
        return math.sqrt(1 + B1 * l2 / (l2 - C1) + B2 * l2 / (l2 - C2) + B3 * l2 / (l2 - C3))


class ACauchyFormula(ARefractiveIndex):
    kind = N.INDEX_CAUCHY

    def __init__(self, A, B, C):
        super().__init__()
        self.par = [float(A), float(B), float(C), 0.0, 0.0, 0.0]

    def coefficients(self):
        return list(self.par)

    def GetRefractiveIndex(self, lam):
        l = lam / 1e-4
        return self.par[0] + self.par[1] * l ** -2 + self.par[2] * l ** -4


class ASchottFormula(ARefractiveIndex):
    kind = N.INDEX_SCHOTT

    def __init__(self, *A):
        super().__init__()
        self.par = [float(a) for a in A]

    def coefficients(self):
        return list(self.par)

    def GetRefractiveIndex(self, lam):
        l = lam / 1e-4
        a = self.par
        return math.sqrt(a[0] + a[1] * l ** 2 + a[2] * l ** -2 + a[3] * l ** -4 + a[4] * l ** -6 + a[5] * l ** -8)


class AMixedRefractiveIndex(ARefractiveIndex):
    kind = N.INDEX_MIXED

    def __init__(self, a: ARefractiveIndex, b: ARefractiveIndex, fa: float, fb: float):
        super().__init__()
        self.a, self.b = a, b
        self.SetFraction(fa, fb)

    def SetFraction(self, fa, fb):
        self.fa, self.fb = fa / (fa + fb), fb / (fa + fb)

    def coefficients(self):
        return [self.fa, self.fb, 0, 0, 0, 0]

    def GetRefractiveIndex(self, lam):
        return self.a.GetRefractiveIndex(lam) * self.fa + self.b.GetRefractiveIndex(lam) * self.fb

    def GetExtinctionCoefficient(self, lam):
        return self.a.GetExtinctionCoefficient(lam) * self.fa + self.b.GetExtinctionCoefficient(lam) * self.fb


def AFilmetrixDotCom(path: str) -> ARefractiveIndex:
    """Filmetrics n,k table: header "Wavelength(nm)<TAB>n<TAB>k", then rows
    (src/AFilmetrixDotCom.cxx)."""
    idx = ARefractiveIndex()
    ng, kg = TGraph(), TGraph()
    with open(path, encoding="utf-8-sig") as f:
        head = f.readline().strip()
        if head != "Wavelength(nm)\tn\tk":
            raise ValueError(f"{path}: invalid data format")
        for line in f:
            parts = line.split()
            if len(parts) < 3:
                continue
            wl, n, k = (float(p) for p in parts[:3])
            ng.SetPoint(ng.GetN(), wl * 1e-7, n)
            kg.SetPoint(kg.GetN(), wl * 1e-7, k)
    idx.SetRefractiveIndex(ng)
    idx.SetExtinctionCoefficient(kg)
    return idx


class AGlassCatalog:
    """Zemax AGF reader: Sellmeier (formula 2) glasses with their internal
    transmittance converted to k (src/AGlassCatalog.cxx:27-107)."""

    def __init__(self, path: str):
        self.index = {}
        name, formula, graph = None, None, None
        with open(path, encoding="latin-1") as f:
            for line in f:
                if line.startswith("NM "):
                    parts = line.split()
                    name = parts[1]
                    try:
                        formula = int(parts[2])
                    except ValueError:
                        formula = int(float(parts[2]))
                    graph = TGraph()
                    self.index[name] = None
                elif line.startswith("CD ") and name is not None:
                    cd = [float(v) for v in line.split()[1:]]
                    if formula == 2 and len(cd) >= 6:
                        s = ASellmeierFormula(cd[0], cd[2], cd[4], cd[1], cd[3], cd[5])
                        s.SetExtinctionCoefficient(graph)
                        self.index[name] = s
                elif line.startswith("IT ") and graph is not None:
                    v = line.split()[1:]
                    if len(v) >= 3:
                        wl, T, d = float(v[0]) * 1e-4, float(v[1]), float(v[2]) * 0.1
                        absl = -d / math.log(T)
                        graph.SetPoint(graph.GetN(), wl, ARefractiveIndex.AbsorptionLengthToExtinctionCoefficient(absl, wl))

    def GetRefractiveIndex(self, name):
        return self.index.get(name)


class AMultilayer:
    """Thin-film stack between a top (incident) and a bottom medium
    (src/AMultilayer.cxx:106-114, 216-238).  Reflectance/transmittance are
    evaluated by the native coherent transfer-matrix code, per ray on the
    GPU when used in a border condition."""

    kS, kP = 0, 1

    def __init__(self, top: ARefractiveIndex, bottom: ARefractiveIndex):
        self.layers = [(top, math.inf, False), (bottom, math.inf, False)]
        self.precalc = None

    def PreCalculateCoherentTMM(self, lam_nbins, lam_min, lam_max, th_nbins, th_min, th_max):
        """Tabulate CoherentTMMMixed at the centres of a lam_nbins x th_nbins
        grid; traces then interpolate the table (TH2::Interpolate) instead
        of evaluating the stack per ray (include/AMultilayer.h:243-262).
        The table is computed on the GPU when the scene is uploaded."""
        self.precalc = (1, int(lam_nbins), float(lam_min), float(lam_max), int(th_nbins), float(th_min),
                        float(th_max))

    def PreCalculateIncoherentTMM(self, lam_nbins, lam_min, lam_max, th_nbins, th_min, th_max):
        """As PreCalculateCoherentTMM with IncoherentTMMMixed values
        (include/AMultilayer.h:263-282)."""
        self.precalc = (2, int(lam_nbins), float(lam_min), float(lam_max), int(th_nbins), float(th_min),
                        float(th_max))

    def AddLayer(self, idx, thickness, coherent=True):
        self.layers.insert(1, (idx, float(thickness), coherent))

    def InsertLayer(self, idx, thickness, coherent=True):
        self.layers.insert(len(self.layers) - 1, (idx, float(thickness), coherent))

    def ChangeThickness(self, i, thickness):
        if i < 1 or i > len(self.layers) - 2:
            raise IndexError(f"cannot change the thickness of layer {i}")
        idx, _, c = self.layers[i]
        self.layers[i] = (idx, float(thickness), c)

    def GetThickness(self, i):
        return self.layers[i][1]

    # -- evaluation (src/AMultilayer.cxx:240-731, include/AMultilayer.h:114-225) --
    # Every call below runs on the GPU through rbg_multilayer_rt, in FP64.
    # Angles may be complex; wavelengths are in the unit of the thicknesses.
    # Reflectance and transmittance are returned, and also stored into
    # ctypes.c_double out-arguments (or list-like ones for the vector forms)
    # when given, as the reference's PyROOT calls pass them.
    def _state(self):
        return (tuple((id(ix), d, c) for ix, d, c in self.layers), self.precalc)

    def _scene(self, reverse=False):
        """(scene, multilayer id) of a one-mirror scene whose border
        condition holds this stack (reversed: the layers bottom to top,
        which is CoherentTMM's `reverse`); rebuilt when the stack changes."""
        key = (self._state(), bool(reverse))
        cache = self.__dict__.setdefault("_scenes", {})
        if key not in cache:
            from .manager import AOpticsManager

            ml = self
            if reverse:
                ml = AMultilayer(self.layers[-1][0], self.layers[0][0])
                ml.layers = list(reversed(self.layers))
            man = AOpticsManager("multilayer", "multilayer evaluation")
            world = AOpticalComponent("world", TGeoBBox("world_box", 10.0, 10.0, 10.0))
            man.SetTopVolume(world)
            mirror = AMirror("coating", TGeoBBox("coating_box", 1.0, 1.0, 1.0))
            world.AddNode(mirror, 1)
            ABorderSurfaceCondition(world, mirror).SetMultilayer(ml)
            scene = man.CloseGeometry()
            cache.clear()
            cache[key] = (man, scene, scene.builder.multilayer_ids[id(ml)])
        _, scene, mid = cache[key]
        return scene, mid

    def _eval(self, mode, pol, th, lam, reverse=False):
        import torch

        scene, mid = self._scene(reverse)
        th = np.atleast_1d(np.asarray(th, dtype=complex))
        lam = np.atleast_1d(np.asarray(lam, dtype=float))
        th, lam = np.broadcast_arrays(th, lam)
        n = th.size
        dev = torch.device("cuda", torch.cuda.current_device())
        t_re = torch.tensor(np.ascontiguousarray(th.real.ravel()), dtype=torch.float64, device=dev)
        t_im = torch.tensor(np.ascontiguousarray(th.imag.ravel()), dtype=torch.float64, device=dev)
        lv = torch.tensor(np.ascontiguousarray(lam.ravel()), dtype=torch.float64, device=dev)
        R = torch.empty(n, dtype=torch.float64, device=dev)
        T = torch.empty(n, dtype=torch.float64, device=dev)
        st = torch.cuda.current_stream().cuda_stream
        N.check(N.lib().rbg_multilayer_rt(scene.handle, mid, mode, pol, n, t_re.data_ptr(), t_im.data_ptr(),
                                          lv.data_ptr(), R.data_ptr(), T.data_ptr(), C.c_void_p(st)),
                "rbg_multilayer_rt")
        return R.cpu().numpy(), T.cpu().numpy()

    @staticmethod
    def _out(scalar, R, T, reflectance, transmittance):
        if scalar:
            r, t = float(R[0]), float(T[0])
            for o, v in ((reflectance, r), (transmittance, t)):
                if o is not None:
                    o.value = v
            return r, t
        for o, v in ((reflectance, R), (transmittance, T)):
            if o is not None:
                if hasattr(o, "clear"):
                    o.clear()
                for x in v:
                    (o.append if hasattr(o, "append") else o.push_back)(float(x))
        return R, T

    def CoherentTMM(self, polarization, th_0, lam_vac, reflectance=None, transmittance=None, reverse=False):
        """R and T of one polarisation (kS, kP); `reverse` traverses the
        stack from the bottom (src/AMultilayer.cxx:240-481)."""
        R, T = self._eval(0, int(polarization), th_0, lam_vac, reverse)
        return self._out(True, R, T, reflectance, transmittance)

    def CoherentTMMS(self, th_0, lam_vac, reflectance=None, transmittance=None):
        return self.CoherentTMM(self.kS, th_0, lam_vac, reflectance, transmittance)

    def CoherentTMMP(self, th_0, lam_vac, reflectance=None, transmittance=None):
        return self.CoherentTMM(self.kP, th_0, lam_vac, reflectance, transmittance)

    def CoherentTMMMixed(self, th_0, lam_vac, reflectance=None, transmittance=None):
        """Mean of p and s, or the precalculated table when one was declared
        (include/AMultilayer.h:114-131).  Either argument may be a sequence
        (the reference's vector overloads, :132-225); the results are then
        arrays."""
        scalar = np.ndim(th_0) == 0 and np.ndim(lam_vac) == 0 and not hasattr(th_0, "__len__") \
            and not hasattr(lam_vac, "__len__")
        R, T = self._eval(2, 2, list(th_0) if hasattr(th_0, "__len__") else th_0,
                          list(lam_vac) if hasattr(lam_vac, "__len__") else lam_vac)
        return self._out(scalar, R, T, reflectance, transmittance)

    def IncoherentTMM(self, polarization, th_0, lam_vac, reflectance=None, transmittance=None):
        """R and T of one polarisation with incoherent layers
        (src/AMultilayer.cxx:555-731)."""
        R, T = self._eval(1, int(polarization), th_0, lam_vac)
        return self._out(True, R, T, reflectance, transmittance)

    def IncoherentTMMS(self, th_0, lam_vac, reflectance=None, transmittance=None):
        return self.IncoherentTMM(self.kS, th_0, lam_vac, reflectance, transmittance)

    def IncoherentTMMP(self, th_0, lam_vac, reflectance=None, transmittance=None):
        return self.IncoherentTMM(self.kP, th_0, lam_vac, reflectance, transmittance)

    def IncoherentTMMMixed(self, th_0, lam_vac, reflectance=None, transmittance=None):
        """Mean of p and s, or the precalculated table when one was declared
        (include/AMultilayer.h:133-149)."""
        mode = 2 if self.precalc is not None else 1
        R, T = self._eval(mode, 2, th_0, lam_vac)
        return self._out(True, R, T, reflectance, transmittance)


# ---------------------------------------------------------------------------
# volumes
# ---------------------------------------------------------------------------
class TGeoVolume:
    """A plain volume (not an optical component): kOther in the reference's
    classification (include/AOpticsManager.h:45-53)."""

    kind = N.KIND_OTHER

    def __init__(self, name: str, shape: TGeoShape, medium=None):
        self.name = name
        self.shape = shape
        self.nodes = []  # (volume, copy_no, matrix, overlap)
        self.conditions: List["ABorderSurfaceCondition"] = []

    def AddNode(self, vol: "TGeoVolume", copy_no: int = 1, matrix: Optional[TGeoMatrix] = None):
        self.nodes.append((vol, int(copy_no), matrix, False))

    def AddNodeOverlap(self, vol: "TGeoVolume", copy_no: int = 1, matrix: Optional[TGeoMatrix] = None):
        self.nodes.append((vol, int(copy_no), matrix, True))

    def GetName(self):
        return self.name

    def GetShape(self):
        return self.shape


class AOpticalComponent(TGeoVolume):
    kind = N.KIND_OPT

    def AddBorderSurfaceCondition(self, condition: "ABorderSurfaceCondition"):
        self.conditions.append(condition)

    def FindBorderSurfaceCondition(self, component2):
        for c in self.conditions:
            if c.component2 is component2:
                return c
        return None


class AMirror(AOpticalComponent):
    kind = N.KIND_MIRROR

    def __init__(self, name, shape, medium=None):
        super().__init__(name, shape, medium)
        self.reflectance = 1.0
        self.reflectance_table = None

    def SetReflectance(self, ref):
        if isinstance(ref, (int, float)):
            self.reflectance = float(ref)
            self.reflectance_table = None
        else:
            self.reflectance_table = ref

    def GetReflectance(self, lam, angle):
        """AMirror::GetReflectance (src/AMirror.cxx:39-60)."""
        t = self.reflectance_table
        if t is None:
            ret = self.reflectance
        elif isinstance(t, TGraph):
            ret = t.Eval(lam)
        else:
            ret = t.Interpolate(lam, angle)
        return min(max(ret, 0.0), 1.0)


class ALens(AOpticalComponent):
    kind = N.KIND_LENS

    def __init__(self, name, shape, medium=None):
        super().__init__(name, shape, medium)
        self.index: Optional[ARefractiveIndex] = None

    def SetRefractiveIndex(self, idx: ARefractiveIndex):
        self.index = idx

    def GetRefractiveIndex(self, lam):
        return self.index.GetRefractiveIndex(lam) if self.index is not None else 1.0

    def GetExtinctionCoefficient(self, lam):
        return self.index.GetExtinctionCoefficient(lam) if self.index is not None else 0.0

    def GetAbsorptionLength(self, lam):
        return self.index.GetAbsorptionLength(lam) if self.index is not None else math.inf


class AFocalSurface(AOpticalComponent):
    kind = N.KIND_FOCUS

    def __init__(self, name, shape, medium=None):
        super().__init__(name, shape, medium)
        self.qe_lambda: Optional[TGraph] = None
        self.qe_angle: Optional[TGraph] = None

    def SetQuantumEfficiency(self, g: TGraph):
        self.qe_lambda = g

    def SetQuantumEfficiencyAngle(self, g: TGraph):
        self.qe_angle = g

    def HasQEAngle(self):
        return self.qe_angle is not None

    def GetQuantumEfficiency(self, lam, angle=None):
        qe = self.qe_lambda.Eval(lam) if self.qe_lambda is not None else 1.0
        if angle is not None and self.qe_angle is not None:
            qe *= self.qe_angle.Eval(angle)
        return qe


class AObscuration(AOpticalComponent):
    kind = N.KIND_OBS


class ABorderSurfaceCondition:
    """Surface condition on the boundary from component1 into component2
    (include/ABorderSurfaceCondition.h:24-48); registers itself on
    component1 (src/ABorderSurfaceCondition.cxx:20-31)."""

    def __init__(self, component1: Optional[AOpticalComponent], component2: Optional[AOpticalComponent]):
        self.component1, self.component2 = component1, component2
        self.sigma = 0.0
        self.multilayer: Optional[AMultilayer] = None
        self.lambertian = False
        if component1 is not None:
            component1.AddBorderSurfaceCondition(self)

    def GetComponent1(self):
        return self.component1

    def GetComponent2(self):
        return self.component2

    def SetGaussianRoughness(self, sigma):
        self.sigma = abs(float(sigma))

    def GetGaussianRoughness(self):
        return self.sigma

    def SetMultilayer(self, m: AMultilayer):
        self.multilayer = m

    def GetMultilayer(self):
        return self.multilayer

    def EnableLambertian(self, enable: bool):
        self.lambertian = bool(enable)

    def IsLambertian(self):
        return self.lambertian


def data_path(*parts):
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), *parts)
