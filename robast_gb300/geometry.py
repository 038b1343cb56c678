"""TGeo-style matrices and shapes used to describe an optical system.

These mirror the ROOT classes that ROBAST scenes are built from
(TGeoTranslation, TGeoRotation, TGeoCombiTrans, TGeoBBox, TGeoTube,
TGeoSphere, TGeoParaboloid, TGeoPgon, TGeoPcon, TGeoCone,
TGeoCompositeShape) and ROBAST's own AGeoAsphericDisk
(include/AGeoAsphericDisk.h:26-122) and AGeoWinstonConePoly
(include/AGeoWinstonConePoly.h:20-63).  They only record parameters; the
scene flattener in the native library turns them into device tables.

Conventions follow TGeo: lengths in cm, angles of constructors in degrees,
matrices map local to master coordinates (master = R local + t).
"""
from __future__ import annotations

import math
import re
from typing import Dict, Optional

import numpy as np

from . import _native as N

# ---------------------------------------------------------------------------
# matrices
# ---------------------------------------------------------------------------
_REGISTRY: Dict[str, "TGeoMatrix"] = {}
_SHAPES: Dict[str, "TGeoShape"] = {}


def euler_matrix(phi: float, theta: float, psi: float) -> np.ndarray:
    """TGeoRotation(phi, theta, psi) (degrees): R = Rz(phi) Rx(theta) Rz(psi)."""
    f, t, p = (math.radians(a) for a in (phi, theta, psi))

    def rz(a):
        c, s = math.cos(a), math.sin(a)
        return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])

    c, s = math.cos(t), math.sin(t)
    rx = np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])
    return rz(f) @ rx @ rz(p)


class TGeoMatrix:
    """Rigid transform master = R @ local + t."""

    def __init__(self, name: str = ""):
        self.name = name
        self.R = np.eye(3)
        self.t = np.zeros(3)

    def RegisterYourself(self):
        if self.name:
            _REGISTRY[self.name] = self
        return self

    def LocalToMaster(self, local):
        return self.R @ np.asarray(local, dtype=float) + self.t

    def LocalToMasterVect(self, local):
        return self.R @ np.asarray(local, dtype=float)

    def MasterToLocal(self, master):
        return self.R.T @ (np.asarray(master, dtype=float) - self.t)

    def as12(self) -> np.ndarray:
        return np.concatenate([self.R.reshape(-1), self.t])

    def __mul__(self, other: "TGeoMatrix") -> "TGeoHMatrix":
        h = TGeoHMatrix()
        h.R = self.R @ other.R
        h.t = self.R @ other.t + self.t
        return h

    def Inverse(self) -> "TGeoHMatrix":
        h = TGeoHMatrix()
        h.R = self.R.T.copy()
        h.t = -self.R.T @ self.t
        return h


class TGeoHMatrix(TGeoMatrix):
    def __init__(self, name: str = "", R=None, t=None):
        super().__init__(name)
        if R is not None:
            self.R = np.asarray(R, dtype=float).reshape(3, 3).copy()
        if t is not None:
            self.t = np.asarray(t, dtype=float).reshape(3).copy()


class TGeoTranslation(TGeoMatrix):
    def __init__(self, *args):
        name = args[0] if args and isinstance(args[0], str) else ""
        vals = args[1:] if name or (args and isinstance(args[0], str)) else args
        super().__init__(name)
        if len(vals) == 3:
            self.t = np.array(vals, dtype=float)

    def SetTranslation(self, x, y, z):
        self.t = np.array([x, y, z], dtype=float)


class TGeoRotation(TGeoMatrix):
    def __init__(self, *args):
        name = args[0] if args and isinstance(args[0], str) else ""
        vals = args[1:] if args and isinstance(args[0], str) else args
        super().__init__(name)
        if len(vals) == 3:
            self.SetAngles(*vals)

    def SetAngles(self, phi, theta, psi):
        self.R = euler_matrix(phi, theta, psi)

    def SetMatrix(self, m):
        self.R = np.asarray(m, dtype=float).reshape(3, 3).copy()

    def _rot_axis(self, axis, deg):
        a = math.radians(deg)
        c, s = math.cos(a), math.sin(a)
        if axis == 0:
            m = np.array([[1, 0, 0], [0, c, -s], [0, s, c]], dtype=float)
        elif axis == 1:
            m = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], dtype=float)
        else:
            m = np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]], dtype=float)
        self.R = m @ self.R

    def RotateX(self, deg):
        self._rot_axis(0, deg)

    def RotateY(self, deg):
        self._rot_axis(1, deg)

    def RotateZ(self, deg):
        self._rot_axis(2, deg)

    def MultiplyBy(self, rot: "TGeoMatrix", after: bool = True):
        """this = this * rot (after) or rot * this."""
        self.R = self.R @ rot.R if after else rot.R @ self.R


class TGeoCombiTrans(TGeoMatrix):
    def __init__(self, *args):
        super().__init__("")
        if args and isinstance(args[0], str):
            self.name = args[0]
            args = args[1:]
        if len(args) == 2 and isinstance(args[0], TGeoMatrix):
            self.t = args[0].t.copy()
            self.R = args[1].R.copy() if args[1] is not None else np.eye(3)
        elif len(args) == 4:
            self.t = np.array(args[:3], dtype=float)
            self.R = args[3].R.copy() if args[3] is not None else np.eye(3)


# ---------------------------------------------------------------------------
# shapes
# ---------------------------------------------------------------------------
class TGeoShape:
    type_id = 0

    def __init__(self, name: str = ""):
        self.name = name
        if name:
            _SHAPES[name] = self

    def params(self) -> list:
        raise NotImplementedError

    def GetName(self):
        return self.name


def _split_name(args, n):
    if args and isinstance(args[0], str):
        return args[0], list(args[1:])
    return "", list(args)


class TGeoBBox(TGeoShape):
    type_id = N.SHAPE_BOX

    def __init__(self, *args):
        name, v = _split_name(args, 3)
        super().__init__(name)
        self.dx, self.dy, self.dz = (float(a) for a in v[:3])
        self.origin = np.array(v[3], dtype=float) if len(v) > 3 and v[3] is not None else np.zeros(3)

    def params(self):
        return [self.dx, self.dy, self.dz, *self.origin]

    def GetDX(self):
        return self.dx

    def GetDY(self):
        return self.dy

    def GetDZ(self):
        return self.dz

    def GetOrigin(self):
        return self.origin


class TGeoTube(TGeoShape):
    type_id = N.SHAPE_TUBE

    def __init__(self, *args):
        name, v = _split_name(args, 3)
        super().__init__(name)
        self.rmin, self.rmax, self.dz = (float(a) for a in v[:3])
        self.phi1, self.phi2 = 0.0, 360.0

    def params(self):
        return [self.rmin, self.rmax, self.dz, self.phi1, self.phi2]

    def GetDz(self):
        return self.dz


class TGeoTubeSeg(TGeoTube):
    def __init__(self, *args):
        name, v = _split_name(args, 5)
        super().__init__(name, *v[:3])
        self.phi1, self.phi2 = float(v[3]), float(v[4])


class TGeoSphere(TGeoShape):
    type_id = N.SHAPE_SPHERE

    def __init__(self, *args):
        name, v = _split_name(args, 2)
        super().__init__(name)
        vals = [0.0, 0.0, 0.0, 180.0, 0.0, 360.0]
        for i, a in enumerate(v[:6]):
            vals[i] = float(a)
        self.rmin, self.rmax, self.theta1, self.theta2, self.phi1, self.phi2 = vals

    def params(self):
        return [self.rmin, self.rmax, self.theta1, self.theta2, self.phi1, self.phi2]


class TGeoParaboloid(TGeoShape):
    type_id = N.SHAPE_PARABOLOID

    def __init__(self, *args):
        name, v = _split_name(args, 3)
        super().__init__(name)
        self.rlo, self.rhi, self.dz = (float(a) for a in v[:3])

    def params(self):
        return [self.rlo, self.rhi, self.dz]


class TGeoPcon(TGeoShape):
    type_id = N.SHAPE_PCON

    def __init__(self, *args):
        name, v = _split_name(args, 3)
        super().__init__(name)
        self.phi1, self.dphi = float(v[0]), float(v[1])
        self.nz = int(v[-1])
        self.z = [0.0] * self.nz
        self.rmin = [0.0] * self.nz
        self.rmax = [0.0] * self.nz

    def DefineSection(self, i, z, rmin, rmax):
        self.z[i], self.rmin[i], self.rmax[i] = float(z), float(rmin), float(rmax)

    def params(self):
        return [self.phi1, self.dphi, self.nz, *self.z, *self.rmin, *self.rmax]


class TGeoPgon(TGeoPcon):
    type_id = N.SHAPE_PGON

    def __init__(self, *args):
        name, v = _split_name(args, 4)
        TGeoShape.__init__(self, name)
        self.phi1, self.dphi, self.nedges, self.nz = float(v[0]), float(v[1]), int(v[2]), int(v[3])
        self.z = [0.0] * self.nz
        self.rmin = [0.0] * self.nz
        self.rmax = [0.0] * self.nz

    def params(self):
        return [self.phi1, self.dphi, self.nedges, self.nz, *self.z, *self.rmin, *self.rmax]


class TGeoCone(TGeoPcon):
    """TGeoCone(dz, rmin1, rmax1, rmin2, rmax2) as a two-section polycone."""

    def __init__(self, *args):
        name, v = _split_name(args, 5)
        TGeoShape.__init__(self, name)
        dz, rmin1, rmax1, rmin2, rmax2 = (float(a) for a in v[:5])
        self.phi1, self.dphi, self.nz = 0.0, 360.0, 2
        self.z, self.rmin, self.rmax = [-dz, dz], [rmin1, rmin2], [rmax1, rmax2]


class _BezierSections:
    """Side surface of AGeoBezierPcon / AGeoBezierPgon
    (src/AGeoBezierPcon.cxx:35-80, src/AGeoBezierPgon.cxx:45-104): the nz
    sections sample a Bezier curve B(t), t = i / (nz - 1), from (0, 0) to
    (1, 1) through 0, 1 or 2 control points, mapped to r = r2 + B.x (r1 - r2)
    and z = -dz + 2 dz B.y; section i is (z, rmin = 0, rmax = r)."""

    def _bezier_init(self, r1, r2, dz):
        self.fLength = 2.0 * float(dz)
        self.fR1, self.fR2 = float(r1), float(r2)
        self.fNcontrol = 0
        self.fP1 = (0.0, 0.0)
        self.fP2 = (0.0, 0.0)

    def Bezier(self, t):
        t = float(t)
        if self.fNcontrol == 0:
            bx, by = t, t
        elif self.fNcontrol == 1:
            a, b, c = (1 - t) * (1 - t), 2 * (1 - t) * t, t * t
            bx, by = b * self.fP1[0] + c, b * self.fP1[1] + c
        else:
            a, b, c, d = (1 - t) ** 3, 3 * (1 - t) * (1 - t) * t, 3 * (1 - t) * t * t, t ** 3
            bx = b * self.fP1[0] + c * self.fP2[0] + d
            by = b * self.fP1[1] + c * self.fP2[1] + d
        return self.fR2 + bx * (self.fR1 - self.fR2), -self.fLength / 2.0 + by * self.fLength

    def SetControlPoints(self, r1, z1, r2=None, z2=None):
        if r2 is None:
            self.fNcontrol, self.fP1, self.fP2 = 1, (float(r1), float(z1)), (0.0, 0.0)
        else:
            self.fNcontrol, self.fP1, self.fP2 = 2, (float(r1), float(z1)), (float(r2), float(z2))
        self.SetSections()

    def SetSections(self):
        for i in range(self.nz):
            r, z = self.Bezier(i / (self.nz - 1))
            self.DefineSection(i, z, 0.0, r)


class AGeoBezierPcon(_BezierSections, TGeoPcon):
    """AGeoBezierPcon([name,] phi, dphi, nz, r1, r2, dz): a polycone whose
    side follows a Bezier curve from radius r2 at -dz to r1 at +dz; the
    sections are set by SetSections / SetControlPoints, as in the reference,
    and the shape is then a plain TGeoPcon."""

    def __init__(self, *args):
        name, v = _split_name(args, 6)
        TGeoPcon.__init__(self, name, v[0], v[1], v[2])
        self._bezier_init(v[3], v[4], v[5])


class AGeoBezierPgon(_BezierSections, TGeoPgon):
    """AGeoBezierPgon([name,] phi, dphi, nedges, nz, r1, r2, dz): the
    polygonal counterpart of AGeoBezierPcon, a plain TGeoPgon once its
    sections are set."""

    def __init__(self, *args):
        name, v = _split_name(args, 7)
        TGeoPgon.__init__(self, name, v[0], v[1], v[2], v[3])
        self._bezier_init(v[4], v[5], v[6])


class AGeoAsphericDisk(TGeoShape):
    """AGeoAsphericDisk(z1, curve1, z2, curve2, rmax, rmin)
    (src/AGeoAsphericDisk.cxx:49-87)."""

    type_id = N.SHAPE_ASPHERIC_DISK

    def __init__(self, *args):
        name, v = _split_name(args, 5)
        super().__init__(name)
        self.z1, self.curve1, self.z2, self.curve2, self.rmax = (float(a) for a in v[:5])
        self.rmin = float(v[5]) if len(v) > 5 else 0.0
        self.conic1 = self.conic2 = 0.0
        self.k1, self.k2 = [], []
        self.steps, self.repeat = 100, 4

    def SetPolynomials(self, n1, k1, n2, k2):
        self.k1 = [float(k1[i]) for i in range(n1)]
        self.k2 = [float(k2[i]) for i in range(n2)]

    def SetConicConstants(self, conic1, conic2):
        self.conic1, self.conic2 = float(conic1), float(conic2)

    def SetFineness(self, steps, repeat):
        if steps > 0:
            self.steps = int(steps)
        if repeat > 0:
            self.repeat = int(repeat)

    def _canon(self):
        z1, c1, z2, c2 = self.z1, self.curve1, self.z2, self.curve2
        if not z1 < z2:
            z1, z2, c1, c2 = z2, z1, c2, c1
        return z1, c1, z2, c2

    def CalcF1(self, r):
        z1, c1, _, _ = self._canon()
        return _asph_sag(r, z1, c1, self.conic1 + 1, self.k1)

    def CalcF2(self, r):
        _, _, z2, c2 = self._canon()
        return _asph_sag(r, z2, c2, self.conic2 + 1, self.k2)

    def params(self):
        return [self.z1, self.curve1, self.z2, self.curve2, self.rmax, self.rmin, self.conic1,
                self.conic2, len(self.k1), len(self.k2), self.steps, self.repeat, *self.k1, *self.k2]


def _asph_sag(r, z0, c, kappa, k):
    p = r * r * c * c * kappa
    if 1 - p < 0:
        raise ValueError("sag undefined at this radius")
    v = z0 + r * r * c / (1 + math.sqrt(1 - p))
    for i, ki in enumerate(k):
        v += ki * r ** (2 * (i + 1))
    return v


class AGeoWinstonConePoly(TGeoShape):
    """AGeoWinstonConePoly(r1, r2, n) (src/AGeoWinstonConePoly.cxx:31-46)."""

    type_id = N.SHAPE_WINSTON_POLY

    def __init__(self, *args):
        name, v = _split_name(args, 3)
        super().__init__(name)
        self.r1, self.r2, self.n = float(v[0]), float(v[1]), int(v[2])

    def GetDZ(self):
        R1, R2 = max(abs(self.r1), abs(self.r2)), min(abs(self.r1), abs(self.r2))
        theta = math.asin(R2 / R1)
        return (R1 + R2) / math.tan(theta) / 2.0

    def params(self):
        return [self.r1, self.r2, self.n]


class AGeoWinstonCone2D(TGeoShape):
    """AGeoWinstonCone2D(r1, r2, y) (src/AGeoWinstonCone2D.cxx:37-51): a
    two-dimensional compound parabolic concentrator, the trough between
    the walls x = +-R(z) of entrance half-width r1 and exit half-width r2,
    extruded over |y| <= y."""

    type_id = N.SHAPE_WINSTON_2D

    def __init__(self, *args):
        name, v = _split_name(args, 3)
        super().__init__(name)
        self.r1, self.r2, self.y = float(v[0]), float(v[1]), float(v[2])

    def GetDZ(self):
        R1, R2 = max(abs(self.r1), abs(self.r2)), min(abs(self.r1), abs(self.r2))
        theta = math.asin(R2 / R1)
        return (R1 + R2) / math.tan(theta) / 2.0

    def GetDY(self):
        return abs(self.y)

    def params(self):
        return [self.r1, self.r2, self.y]


class TGeoCompositeShape(TGeoShape):
    """Boolean shape.  Built either from a ROOT-style expression over named
    shapes and registered matrices ("mirSphere:transZ*mirCut",
    "A:tr1 - B:tr2", "a + b + c") or explicitly with (op, left, right,
    left_matrix, right_matrix)."""

    type_id = N.SHAPE_COMPOSITE
    _OPS = {"+": N.OP_UNION, "*": N.OP_INTERSECTION, "-": N.OP_SUBTRACTION}

    def __init__(self, name: str, expr: Optional[str] = None, *, op=None, left=None, right=None,
                 left_matrix: Optional[TGeoMatrix] = None, right_matrix: Optional[TGeoMatrix] = None):
        super().__init__(name)
        if expr is not None:
            node = _parse_boolean(expr)
            self.op, self.left, self.right, self.left_matrix, self.right_matrix = node
        else:
            self.op, self.left, self.right = op, left, right
            self.left_matrix, self.right_matrix = left_matrix, right_matrix

    def params(self):
        return []


_TOKEN = re.compile(r"\s*([A-Za-z_][A-Za-z0-9_]*|[-+*():])")


def _parse_boolean(expr: str):
    """Parse "a:m1 op b:m2 ..." with * binding tighter than + and -, both
    left-associative, and parentheses.  Returns (op, left, right, lm, rm)
    of the root node."""
    toks = [t for t in _TOKEN.findall(expr)]
    pos = [0]

    def peek():
        return toks[pos[0]] if pos[0] < len(toks) else None

    def take():
        if pos[0] >= len(toks):
            raise ValueError(f"unexpected end of {expr!r}")
        t = toks[pos[0]]
        pos[0] += 1
        return t

    def as_shape(operand):
        shape, mat = operand
        if mat is None:
            return shape
        # a matrix on a whole operand: wrap as union with itself
        c = TGeoCompositeShape.__new__(TGeoCompositeShape)
        TGeoShape.__init__(c, "")
        c.op, c.left, c.right, c.left_matrix, c.right_matrix = N.OP_UNION, shape, shape, mat, mat
        return c

    def primary():
        t = take()
        if t == "(":
            shape = as_shape(expr_())
            if take() != ")":
                raise ValueError(f"unbalanced parentheses in {expr!r}")
        else:
            if t not in _SHAPES:
                raise KeyError(f"unknown shape {t!r} in {expr!r}")
            shape = _SHAPES[t]
        mat = None
        if peek() == ":":
            take()
            m = take()
            if m not in _REGISTRY:
                raise KeyError(f"unregistered matrix {m!r} in {expr!r}")
            mat = _REGISTRY[m]
        return (shape, mat)

    def combine(left, right, op):
        c = TGeoCompositeShape.__new__(TGeoCompositeShape)
        TGeoShape.__init__(c, "")
        c.op, c.left, c.left_matrix = op, left[0], left[1]
        c.right, c.right_matrix = right[0], right[1]
        return (c, None)

    def term():
        left = primary()
        while peek() == "*":
            take()
            left = combine(left, primary(), N.OP_INTERSECTION)
        return left

    def expr_():
        left = term()
        while peek() in ("+", "-"):
            op = N.OP_UNION if take() == "+" else N.OP_SUBTRACTION
            left = combine(left, term(), op)
        return left

    root = expr_()
    if peek() is not None:
        raise ValueError(f"trailing tokens in {expr!r}")
    node = as_shape(root)
    if not isinstance(node, TGeoCompositeShape):
        return N.OP_UNION, node, node, None, None
    return node.op, node.left, node.right, node.left_matrix, node.right_matrix
