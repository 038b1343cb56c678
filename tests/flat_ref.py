"""An independent flattening of a scene description for the FP64 oracle.

The oracle traces the physical node tree of a flattened scene
(rbg_flat_scene).  The product builds that tree in C++ (rbg_scene_create);
if the oracle read the product's output, a flattening error (a matrix
composed in the wrong order, a derived shape constant, a Winston cone's
dimensions) would be invisible to every parity test.  This module derives
the same structure a second time, in Python, straight from the scene
description (rbg_scene_desc, the arrays the Python classes hand to the
library) and from the reference's own definitions:

* the physical tree: TGeoVolume::AddNode placements expanded breadth first,
  a node's daughters numbered consecutively in placement order (the node
  numbering of include/robast_gb.h), local -> master matrices composed as
  TGeoHMatrix products (mother * placement);
* canonical shape parameters (include/robast_gb_layout.h): TGeoTubeSeg /
  TGeoSphere phi ranges as (phi1, dphi); TGeoParaboloid's z = a r^2 + b with
  a = 2 dz / (rhi^2 - rlo^2), b = -dz - a rlo^2; AGeoAsphericDisk's
  SetAsphDimensions (surfaces ordered z1 < z2, |r| ordered), kappa = conic
  + 1, and ComputeBBox's origin and half height from its stepped search
  (src/AGeoAsphericDisk.cxx:164-243, 971-1013), the sags at rmin / rmax;
  AGeoWinstonConePoly::SetWinstonDimensions
  (src/AGeoWinstonConePoly.cxx:356-386) and AGeoWinstonCone2D's
  (src/AGeoWinstonCone2D.cxx:551-567); a composite's two operand matrices;
* conservative master-frame bounding boxes from each shape's own extent.

No BVH is built: the oracle scans a mother's daughters.  Test
infrastructure only.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from robast_gb300 import _native as N

BIG = 1e30
MAX_DEPTH = 64


def _m12(a):
    return np.asarray(a, dtype=np.float64).reshape(12)


def _compose(a, b):
    """TGeoHMatrix product a * b of two 12-double local -> master matrices."""
    Ra, ta = a[:9].reshape(3, 3), a[9:]
    Rb, tb = b[:9].reshape(3, 3), b[9:]
    return np.concatenate([(Ra @ Rb).reshape(-1), Ra @ tb + ta])


IDENTITY = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0], dtype=np.float64)


def _sag(r, z0, c, kappa, k):
    """CalcF1 / CalcF2 (src/AGeoAsphericDisk.cxx:126-153); None where the
    conic is undefined (the reference throws)."""
    p = r * r * c * c * kappa
    if 1 - p < 0:
        return None
    v = z0 + r * r * c / (1 + math.sqrt(1 - p))
    for i, ki in enumerate(k):
        v += ki * r ** (2 * (i + 1))
    return v


def _asph_canonical(u):
    z1, c1, z2, c2, rmax, rmin, conic1, conic2 = u[:8]
    n1, n2, steps, repeat = int(u[8]), int(u[9]), int(u[10]), int(u[11])
    k1 = list(u[12:12 + n1])
    k2 = list(u[12 + n1:12 + n1 + n2])
    if not z1 < z2:
        z1, z2, c1, c2 = z2, z1, c2, c1
    rmax, rmin = abs(rmax), abs(rmin)
    if not rmax > rmin:
        rmax, rmin = rmin, rmax
    kap1, kap2 = conic1 + 1, conic2 + 1
    f1 = lambda r: _sag(r, z1, c1, kap1, k1)
    f2 = lambda r: _sag(r, z2, c2, kap2, k2)

    def extreme(f, n, upper):
        # ComputeBBox: the extreme sag over [rmin, rmax] by a stepped search
        # refined `repeat` times around the best radius (j runs to steps + 1)
        if n == 0:
            a, b = f(rmin), f(rmax)
            if a is None or b is None:
                return BIG if upper else -BIG
            return max(a, b) if upper else min(a, b)
        best = -BIG if upper else BIG
        r1, r2 = rmin, rmax
        for _ in range(repeat):
            step = (r2 - r1) / steps
            rb = r1
            for j in range(steps + 2):
                r = r1 + j * step
                v = f(r)
                if v is None:
                    v = -BIG if upper else BIG
                if (v > best) if upper else (v < best):
                    best, rb = v, r
            r1 = rmin if rb == rmin else rb - step
            r2 = rmax if rb == rmax else rb + step
        return best

    zmax = extreme(f2, n2, True)
    zmin = extreme(f1, n1, False)
    nan = float("nan")

    def at(f, r):
        v = f(r)
        return nan if v is None else v

    return [z1, z2, c1, c2, kap1, kap2, rmin, rmax, n1, n2, (zmax + zmin) / 2, (zmax - zmin) / 2,
            1.0 if rmin > 0 else 0.0, at(f1, rmin), at(f2, rmin), at(f1, rmax), at(f2, rmax)] + k1 + k2


def _winston_canonical(u, two_d):
    r1, r2, third = u[:3]
    R1, R2 = (abs(r1), abs(r2)) if abs(r1) > abs(r2) else (abs(r2), abs(r1))
    theta = math.asin(R2 / R1)
    dz = (R1 + R2) / math.tan(theta) / 2.0
    f = R2 * (1 + math.sin(theta))
    if two_d:
        return [R1, R2, 2, theta, f, dz, R1, abs(third)]
    n = int(third)
    npoly = n if n >= 3 else 3
    # the reference takes the circumradius from the raw r1 and n
    r = r1 / math.cos(math.pi / n)
    dx = max(abs(r * math.cos(math.pi / n * (2 * i + 1))) for i in range(npoly))
    dy = max(abs(r * math.sin(math.pi / n * (2 * i + 1))) for i in range(npoly))
    return [R1, R2, npoly, theta, f, dz, dx, dy]


def _phi_range(phi1, phi2):
    """(phi1, dphi) of TGeoTubeSeg / TGeoSphere: the range runs
    counter-clockwise from phi1 to phi2; a span of 360 deg or more is full."""
    d = phi2 - phi1
    if d >= 360.0:
        return phi1, 360.0
    while d <= 0:
        d += 360.0
    return phi1, d


def canonical_params(stype, u):
    u = list(u)
    if stype == N.SHAPE_BOX:
        return u[:6]
    if stype == N.SHAPE_TUBE:
        p1, d = _phi_range(u[3], u[4])
        return [u[0], u[1], u[2], p1, d]
    if stype == N.SHAPE_SPHERE:
        p1, d = _phi_range(u[4], u[5])
        return [u[0], u[1], u[2], u[3], p1, d]
    if stype == N.SHAPE_PARABOLOID:
        rlo, rhi, dz = u[:3]
        a = 2 * dz / (rhi * rhi - rlo * rlo)
        return [rlo, rhi, dz, a, -dz - a * rlo * rlo]
    if stype in (N.SHAPE_PGON, N.SHAPE_PCON):
        return u
    if stype == N.SHAPE_ASPHERIC_DISK:
        return _asph_canonical(u)
    if stype == N.SHAPE_WINSTON_POLY:
        return _winston_canonical(u, False)
    if stype == N.SHAPE_WINSTON_2D:
        return _winston_canonical(u, True)
    raise ValueError(f"shape type {stype}")


def _angles(phi1, dphi, extra=()):
    """The angles (deg) at which a cos / sin extreme can occur on the arc
    [phi1, phi1 + dphi]: its ends and the axis directions inside it."""
    if dphi >= 360.0:
        return [0.0, 90.0, 180.0, 270.0]
    out = [phi1, phi1 + dphi]
    for a in (0.0, 90.0, 180.0, 270.0) + tuple(extra):
        k = math.ceil((phi1 - a) / 360.0)
        if a + 360.0 * k <= phi1 + dphi:
            out.append(a + 360.0 * k)
    return out


def _xy_box(radii, phis):
    xs = [r * math.cos(math.radians(p)) for r in radii for p in phis]
    ys = [r * math.sin(math.radians(p)) for r in radii for p in phis]
    return min(xs), max(xs), min(ys), max(ys)


def _local_box(stype, P, shapes, pp):
    """Axis-aligned local box (lo, hi) enclosing a shape, from canonical
    parameters: the box of the shape's extreme points (arc ends and axis
    crossings of phi ranges, polygon vertices, theta-range ends)."""
    if stype == N.SHAPE_BOX:
        o = np.array(P[3:6])
        d = np.array(P[0:3])
        return o - d, o + d
    if stype == N.SHAPE_TUBE:
        x0, x1, y0, y1 = _xy_box([P[0], P[1]], _angles(P[3], P[4]))
        return np.array([x0, y0, -P[2]]), np.array([x1, y1, P[2]])
    if stype == N.SHAPE_SPHERE:
        rmin, rmax, t1, t2 = P[0], P[1], P[2], P[3]
        thetas = [t1, t2] + ([90.0] if t1 < 90.0 < t2 else [])
        phis = _angles(P[4], P[5])
        pts = []
        for r in (rmin, rmax):
            for t in thetas + [0.0 if t1 <= 0.0 else t1, 180.0 if t2 >= 180.0 else t2]:
                st, ct = math.sin(math.radians(t)), math.cos(math.radians(t))
                for ph in phis:
                    pts.append((r * st * math.cos(math.radians(ph)), r * st * math.sin(math.radians(ph)), r * ct))
        a = np.array(pts)
        return a.min(axis=0), a.max(axis=0)
    if stype == N.SHAPE_PARABOLOID:
        return np.array([-P[1], -P[1], -P[2]]), np.array([P[1], P[1], P[2]])
    if stype in (N.SHAPE_PGON, N.SHAPE_PCON):
        pg = stype == N.SHAPE_PGON
        nz = int(P[3] if pg else P[2])
        z = P[(4 if pg else 3):][:nz]
        rmin = P[(4 if pg else 3) + nz:][:nz]
        rmax = P[(4 if pg else 3) + 2 * nz:][:nz]
        if pg:
            # polygon vertices at phi1 + k dphi / n, radius apothem / cos(half sector)
            n = int(P[2])
            half = P[1] / n / 2
            phis = [P[0] + k * P[1] / n for k in range(n + 1)]
            radii = [r / math.cos(math.radians(half)) for r in (min(rmin), max(rmax))]
            if P[1] < 360.0:
                radii.append(0.0 if min(rmin) == 0 else min(rmin))
        else:
            phis = _angles(P[0], P[1])
            radii = [min(rmin), max(rmax)]
        x0, x1, y0, y1 = _xy_box(radii, phis)
        return np.array([x0, y0, min(z)]), np.array([x1, y1, max(z)])
    if stype == N.SHAPE_ASPHERIC_DISK:
        r, oz, dz = P[7], P[10], P[11]
        return np.array([-r, -r, oz - dz]), np.array([r, r, oz + dz])
    if stype in (N.SHAPE_WINSTON_POLY, N.SHAPE_WINSTON_2D):
        return np.array([-P[6], -P[7], -P[5]]), np.array([P[6], P[7], P[5]])
    raise ValueError(stype)


def _transform_box(lo, hi, m):
    R, t = m[:9].reshape(3, 3), m[9:]
    c = (lo + hi) / 2
    h = (hi - lo) / 2
    cm = R @ c + t
    hm = np.abs(R) @ h
    return cm - hm, cm + hm


def _pad(lo, hi):
    # generous against rounding: the oracle only culls with these boxes
    e = 1e-7 * np.maximum(1.0, np.maximum(np.abs(lo), np.abs(hi))) + 1e-6
    return lo - e, hi + e


class IndependentFlat:
    """Holds the arrays of an rbg_flat_scene derived from a Scene's
    description; `.flat` is the ctypes struct the oracle reads."""

    def __init__(self, scene):
        d = scene.desc
        shapes = [d.shapes[i] for i in range(d.n_shapes)]
        mats = [_m12([d.matrices[12 * i + k] for k in range(12)]) for i in range(d.n_matrices)]
        user = [d.params[i] for i in range(d.n_params)]
        volumes = [d.volumes[i] for i in range(d.n_volumes)]

        def mat(i):
            return IDENTITY if i < 0 else mats[i]

        # canonical shapes
        pool = []
        canon = {}
        out_shapes = []
        for sid, sh in enumerate(shapes):
            if sh.type == N.SHAPE_COMPOSITE:
                pp = list(mat(sh.left_matrix)) + list(mat(sh.right_matrix))
            else:
                pp = canonical_params(sh.type, user[sh.param_offset:sh.param_offset + sh.n_params])
            canon[sid] = pp
            off = len(pool)
            pool.extend(float(v) for v in pp)
            out_shapes.append(N.ShapeDesc(sh.type, off, len(pp), sh.op, sh.left, sh.right, sh.left_matrix,
                                          sh.right_matrix))
        self.canonical = canon

        # local boxes, composites from their operands
        boxes = {}

        def box(sid):
            if sid in boxes:
                return boxes[sid]
            sh = shapes[sid]
            if sh.type != N.SHAPE_COMPOSITE:
                b = _local_box(sh.type, canon[sid], shapes, canon)
            else:
                la, ha = _transform_box(*box(sh.left), mat(sh.left_matrix))
                lb, hb = _transform_box(*box(sh.right), mat(sh.right_matrix))
                if sh.op == N.OP_UNION:
                    b = (np.minimum(la, lb), np.maximum(ha, hb))
                elif sh.op == N.OP_INTERSECTION:
                    b = (np.maximum(la, lb), np.minimum(ha, hb))
                else:
                    b = (la, ha)
            boxes[sid] = b
            return b

        # physical tree, breadth first
        by_mother = {}
        for i in range(d.n_placements):
            pl = d.placements[i]
            by_mother.setdefault(pl.mother, []).append(pl)
        nodes = [dict(parent=-1, volume=d.top_volume, m=IDENTITY.copy(), depth=0)]
        children = []
        cur = 0
        while cur < len(nodes):
            n = nodes[cur]
            pls = by_mother.get(n["volume"], [])
            first = len(nodes)
            for pl in pls:
                nodes.append(dict(parent=cur, volume=pl.daughter, m=_compose(n["m"], mat(pl.matrix)),
                                  depth=n["depth"] + 1))
                if n["depth"] + 1 >= MAX_DEPTH:
                    raise ValueError("placement tree too deep")
            n["child_begin"] = len(children)
            n["child_count"] = len(pls)
            children.extend(range(first, first + len(pls)))
            cur += 1
        self.nodes_py = nodes
        arr_nodes = (N.Node * len(nodes))()
        for i, n in enumerate(nodes):
            v = volumes[n["volume"]]
            lo, hi = _pad(*_transform_box(*box(v.shape), n["m"]))
            a = arr_nodes[i]
            a.parent, a.volume, a.shape, a.kind = n["parent"], n["volume"], v.shape, v.kind
            a.child_begin, a.child_count, a.bvh_root, a.depth = n["child_begin"], n["child_count"], -1, n["depth"]
            for k in range(12):
                a.m[k] = float(n["m"][k])
            for k in range(3):
                a.lo[k], a.hi[k] = float(lo[k]), float(hi[k])
        self._keep = [arr_nodes, (C.c_int32 * max(1, len(children)))(*children),
                      (N.ShapeDesc * max(1, len(out_shapes)))(*out_shapes),
                      (C.c_double * max(1, len(pool)))(*pool)]
        f = N.FlatScene()
        f.n_nodes, f.nodes = len(nodes), C.cast(self._keep[0], C.POINTER(N.Node))
        f.n_children, f.children = len(children), C.cast(self._keep[1], C.POINTER(C.c_int32))
        f.n_bvh, f.n_bvh_items = 0, 0
        f.n_shapes, f.shapes = len(out_shapes), C.cast(self._keep[2], C.POINTER(N.ShapeDesc))
        # materials, tables and conditions are the description's own tables
        f.n_volumes, f.volumes = d.n_volumes, d.volumes
        f.n_tables, f.tables = d.n_tables, d.tables
        f.n_indices, f.indices = d.n_indices, d.indices
        f.n_layers, f.layers = d.n_layers, d.layers
        f.n_multilayers, f.multilayers = d.n_multilayers, d.multilayers
        f.n_borders, f.borders = d.n_borders, d.borders
        # tables and refractive-index coefficients keep their description
        # offsets into the user pool; shapes point into the canonical pool
        # placed after it
        base = d.n_params
        full = list(user) + [float(v) for v in pool]
        shapes2 = (N.ShapeDesc * max(1, len(out_shapes)))()
        for i, s in enumerate(out_shapes):
            shapes2[i] = N.ShapeDesc(s.type, s.param_offset + base, s.n_params, s.op, s.left, s.right,
                                     s.left_matrix, s.right_matrix)
        self._keep += [shapes2, (C.c_double * max(1, len(full)))(*full)]
        f.shapes = C.cast(shapes2, C.POINTER(N.ShapeDesc))
        f.n_params, f.params = len(full), C.cast(self._keep[-1], C.POINTER(C.c_double))
        f.top_node = 0
        self.flat = f
        self.pool_base = base


def independent_flat(scene):
    """The scene's independent flattening, built once and kept on it."""
    f = getattr(scene, "_independent_flat", None)
    if f is None:
        f = IndependentFlat(scene)
        scene._independent_flat = f
    return f
