"""AOpticsManager, ARay, ARayArray and ARayShooter with ROBAST's API.

``AOpticsManager.TraceNonSequential`` (include/AOpticsManager.h:92-100,
src/AOpticsManager.cxx:327-587) hands the whole ray batch to the GPU through
the C ABI (include/robast_gb.h).  There is no host fallback: if the native
library or the GPU is missing the call raises.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Dict, List, Optional

import numpy as np

from . import _native as N
from .geometry import TGeoCompositeShape, TGeoMatrix, TGeoShape
from .optics import (AFocalSurface, ALens, AMirror, AMultilayer, AObscuration, AOpticalComponent, ARefractiveIndex,
                     TGraph, TGraph2D, TGeoVolume, TH2)

SPEED_OF_LIGHT = 299792458.0  # m/s


# ---------------------------------------------------------------------------
# rays
# ---------------------------------------------------------------------------
class ARay:
    """One ray (src/ARay.cxx).  Status values follow include/ARay.h:26."""

    kRun, kStop, kExit, kFocus, kSuspend, kAbsorb = range(6)

    def __init__(self, id=0, lam=0.0, x=0.0, y=0.0, z=0.0, t=0.0, dx=1.0, dy=0.0, dz=0.0):
        self.id = id
        self.lam = float(lam)
        self.points = [(float(x), float(y), float(z), float(t))]
        self.nodes: List[int] = []
        self.direction = np.zeros(3)
        self.SetDirection(dx, dy, dz)
        self.status = ARay.kRun
        self.npoints = 1
        self.last_node = -2

    def SetDirection(self, dx, dy, dz):
        mag = math.sqrt(dx * dx + dy * dy + dz * dz)
        if mag > 0:
            self.direction = np.array([dx / mag, dy / mag, dz / mag])

    def GetDirection(self, out=None):
        if out is not None:
            out[:3] = list(self.direction)
        return self.direction.copy()

    def GetLastPoint(self, out=None):
        p = self.points[-1]
        if out is not None:
            out[:4] = list(p)
        return np.array(p)

    def GetNpoints(self):
        return self.npoints

    def GetLambda(self):
        return self.lam

    def IsAbsorbed(self):
        return self.status == ARay.kAbsorb

    def IsExited(self):
        return self.status == ARay.kExit

    def IsFocused(self):
        return self.status == ARay.kFocus

    def IsRunning(self):
        return self.status == ARay.kRun

    def IsStopped(self):
        return self.status == ARay.kStop

    def IsSuspended(self):
        return self.status == ARay.kSuspend

    def GetPoint(self, i):
        """Point i (x, y, z, t); the start point is point 0."""
        return np.array(self.points[i])

    def SetLambda(self, lam):
        self.lam = float(lam)

    # fate setters (include/ARay.h:47-52)
    def Absorb(self):
        self.status = ARay.kAbsorb

    def Exit(self):
        self.status = ARay.kExit

    def Focus(self):
        self.status = ARay.kFocus

    def Stop(self):
        self.status = ARay.kStop

    def Suspend(self):
        self.status = ARay.kSuspend

    def FindNode(self, name: str):
        """The node of the history named exactly `name` ("<volume>_<copy>"),
        None if none (include/ARay.h:46-48, TObjArray::FindObject)."""
        names = getattr(self, "node_names", None) or []
        for nd in self.nodes:
            if 0 <= nd < len(names) and names[nd] == name:
                return name
        return None

    def GetNodeHistory(self):
        """Physical node ids of the history (-1: outside the top volume)."""
        return list(self.nodes)

    def FindNodeNumberStartWith(self, name: str) -> int:
        """Index in the node history of the first node whose TGeoNode name
        starts with `name`, -1 if none (src/ARay.cxx:55-64).  Node i of the
        history was added together with point i + 1."""
        names = getattr(self, "node_names", None) or []
        for i, nd in enumerate(self.nodes):
            if 0 <= nd < len(names) and names[nd].startswith(name):
                return i
        return -1

    def FindNodeStartWith(self, name: str):
        """Name of that node, None if none (src/ARay.cxx:42-53)."""
        i = self.FindNodeNumberStartWith(name)
        return None if i < 0 else self.node_names[self.nodes[i]]


class ARayArray:
    """Batch of rays as structure-of-arrays.  After tracing, rays are binned
    by status like the reference (src/ARayArray.cxx:41-56): GetFocused() etc.
    return index arrays into the batch."""

    _FIELDS = ("x", "y", "z", "t", "dx", "dy", "dz", "lam")

    def __init__(self, n: int = 0):
        for f in self._FIELDS:
            setattr(self, f, np.zeros(n))
        self.status = np.zeros(n, dtype=np.uint8)
        self.npoints = np.ones(n, dtype=np.int32)
        self.last_node = np.full(n, -2, dtype=np.int32)
        self.hist_xyzt = None
        self.hist_node = None
        self.node_names: List[str] = []
        self._pending: List[ARay] = []

    @classmethod
    def from_arrays(cls, x, y, z, dx, dy, dz, lam, t=None):
        a = cls(0)
        n = len(x)
        a.x, a.y, a.z = (np.ascontiguousarray(v, dtype=float) for v in (x, y, z))
        a.dx, a.dy, a.dz = (np.ascontiguousarray(v, dtype=float) for v in (dx, dy, dz))
        a.lam = np.ascontiguousarray(np.broadcast_to(np.asarray(lam, dtype=float), (n,)))
        a.t = np.zeros(n) if t is None else np.ascontiguousarray(t, dtype=float)
        a.status = np.zeros(n, dtype=np.uint8)
        a.npoints = np.ones(n, dtype=np.int32)
        a.last_node = np.full(n, -2, dtype=np.int32)
        return a

    def Add(self, ray: ARay):
        self._pending.append(ray)

    def _flush(self):
        if not self._pending:
            return
        rays = self._pending
        self._pending = []
        extra = ARayArray.from_arrays([r.points[-1][0] for r in rays], [r.points[-1][1] for r in rays],
                                      [r.points[-1][2] for r in rays], [r.direction[0] for r in rays],
                                      [r.direction[1] for r in rays], [r.direction[2] for r in rays],
                                      [r.lam for r in rays], [r.points[-1][3] for r in rays])
        for f in self._FIELDS + ("status", "npoints", "last_node"):
            setattr(self, f, np.concatenate([getattr(self, f), getattr(extra, f)]))

    def __len__(self):
        self._flush()
        return len(self.x)

    def _bin(self, st):
        self._flush()
        return np.nonzero(self.status == st)[0]

    def GetAbsorbed(self):
        return self._bin(N.RBG_ABSORB)

    def GetExited(self):
        return self._bin(N.RBG_EXIT)

    def GetFocused(self):
        return self._bin(N.RBG_FOCUS)

    def GetRunning(self):
        return self._bin(N.RBG_RUN)

    def GetStopped(self):
        return self._bin(N.RBG_STOP)

    def GetSuspended(self):
        return self._bin(N.RBG_SUSPEND)

    def points(self, idx=None):
        """Last points (x, y, z, t) of the selected rays."""
        self._flush()
        sel = slice(None) if idx is None else idx
        return np.stack([self.x[sel], self.y[sel], self.z[sel], self.t[sel]], axis=-1)

    def directions(self, idx=None):
        self._flush()
        sel = slice(None) if idx is None else idx
        return np.stack([self.dx[sel], self.dy[sel], self.dz[sel]], axis=-1)

    # -- per-ray histories (TraceNonSequential(..., history=H)) ------------
    def _need_history(self):
        if self.hist_node is None:
            raise RuntimeError("no point/node history: trace with history > 0")

    def GetPoint(self, i, n):
        """Point n (x, y, z, t) of ray i; the start point is point 0.
        Points past the traced history capacity were not kept (NaN)."""
        self._need_history()
        if n < 0 or n >= min(int(self.npoints[i]), self.hist_xyzt.shape[1]):
            return np.full(4, np.nan)
        return self.hist_xyzt[i, n].copy()

    def GetNodeHistory(self, i):
        """Physical node ids of ray i in ARay::fNodeHisotry order (node k was
        added with point k + 1; -1 is a null node outside the top volume)."""
        self._need_history()
        m = min(int(self.npoints[i]), self.hist_node.shape[1])
        return self.hist_node[i, 1:m].copy()

    def FindNodeNumberStartWith(self, name: str, idx=None):
        """ARay::FindNodeNumberStartWith for every selected ray at once
        (src/ARay.cxx:55-64): the history index of the first node whose
        TGeoNode name ("<volume>_<copy>") starts with `name`, -1 if none."""
        self._need_history()
        names = self.node_names
        match = np.array([nm.startswith(name) for nm in names] + [False], dtype=bool)
        sel = slice(None) if idx is None else idx
        hn = self.hist_node[sel, 1:]
        npts = self.npoints[sel]
        k = np.arange(hn.shape[1])
        valid = (k[None, :] < (npts[:, None] - 1)) & (hn >= 0)
        hit = valid & match[np.where(valid, hn, len(names))]
        first = np.argmax(hit, axis=1)
        return np.where(hit.any(axis=1), first, -1).astype(np.int64)

    def FindNodeStartWith(self, name: str, idx=None):
        """Physical node id of that node per selected ray, -1 if none
        (src/ARay.cxx:42-53 returns the TGeoNode; node_names maps ids to
        names)."""
        k = self.FindNodeNumberStartWith(name, idx)
        sel = slice(None) if idx is None else idx
        hn = self.hist_node[sel, 1:]
        rows = np.arange(len(k))
        return np.where(k >= 0, hn[rows, np.maximum(k, 0)], -1).astype(np.int32)

    def NodeHitPoints(self, name: str, idx=None):
        """For every selected ray whose history holds a node starting with
        `name`: (ray index, the point recorded with that node).  The hit map
        of tutorials/DaviesCotton.C:214-223 (GetPoint of the first
        "mirror" node), with the point the node was added with."""
        sel_idx = np.arange(len(self)) if idx is None else np.asarray(idx)
        k = self.FindNodeNumberStartWith(name, sel_idx)
        ok = k >= 0
        rows = sel_idx[ok]
        return rows, self.hist_xyzt[rows, k[ok] + 1]

    def Merge(self, other: "ARayArray"):
        self._flush()
        other._flush()
        for f in self._FIELDS + ("status", "npoints", "last_node"):
            setattr(self, f, np.concatenate([getattr(self, f), getattr(other, f)]))

    def rays_struct(self):
        """ctypes rbg_rays over this batch (host pointers, kept alive by self)."""
        self._flush()
        dp = C.POINTER(C.c_double)
        for f in self._FIELDS:
            setattr(self, f, np.ascontiguousarray(getattr(self, f), dtype=np.float64))
        return N.Rays(len(self.x), *(getattr(self, f).ctypes.data_as(dp) for f in self._FIELDS))


# ---------------------------------------------------------------------------
# ray sources (src/ARayShooter.cxx)
# ---------------------------------------------------------------------------
class ARayShooter:
    seed = 0x5EED0001

    @staticmethod
    def _shoot(kind, params, n, lam, rot, tr, v, seed=None, first_id=0):
        cap = n
        out = ARayArray(cap)
        dp = C.POINTER(C.c_double)
        rays = N.Rays(cap, *(getattr(out, f).ctypes.data_as(dp) for f in ARayArray._FIELDS))
        p = (C.c_double * max(1, len(params)))(*params)
        r9 = (C.c_double * 9)(*rot.R.reshape(-1)) if rot is not None else None
        t3 = (C.c_double * 3)(*tr.t) if tr is not None else None
        if v is not None:
            vv = np.asarray([v[0], v[1], v[2]] if not hasattr(v, "X") else [v.X(), v.Y(), v.Z()], dtype=float)
            d3 = (C.c_double * 3)(*vv)
        else:
            d3 = None
        s = ARayShooter.seed if seed is None else seed
        N.check(N.lib().rbg_shoot(kind, p, n, r9, t3, d3, s, first_id, lam, C.byref(rays)), "rbg_shoot")
        m = rays.n
        for f in ARayArray._FIELDS:
            setattr(out, f, getattr(out, f)[:m].copy())
        out.status = out.status[:m].copy()
        out.npoints = out.npoints[:m].copy()
        out.last_node = out.last_node[:m].copy()
        return out

    @staticmethod
    def Circle(lam, rmax, nr, nphi, rot=None, tr=None, v=None):
        n = 1 + nphi * nr * (nr + 1) // 2
        return ARayShooter._shoot(N.RBG_SHOOT_CIRCLE, [rmax, nr, nphi],
                                  n, lam, rot, tr, v)

    @staticmethod
    def RandomCircle(lam, rmax, n, rot=None, tr=None, v=None, seed=None, first_id=0):
        return ARayShooter._shoot(N.RBG_SHOOT_RANDOM_CIRCLE, [rmax], n, lam, rot, tr, v, seed, first_id)

    @staticmethod
    def RandomCone(lam, r, d, n, rot=None, tr=None, seed=None, first_id=0):
        return ARayShooter._shoot(N.RBG_SHOOT_RANDOM_CONE, [r, d], n, lam, rot, tr, None, seed, first_id)

    @staticmethod
    def RandomRectangle(lam, dx, dy, n, rot=None, tr=None, v=None, seed=None, first_id=0):
        return ARayShooter._shoot(N.RBG_SHOOT_RANDOM_RECTANGLE, [dx, dy], n, lam, rot, tr, v, seed, first_id)

    @staticmethod
    def RandomSphere(lam, n, tr=None, seed=None, first_id=0):
        return ARayShooter._shoot(N.RBG_SHOOT_RANDOM_SPHERE, [0.0], n, lam, None, tr, None, seed, first_id)

    @staticmethod
    def RandomSphericalCone(lam, n, theta, rot=None, tr=None, seed=None, first_id=0):
        return ARayShooter._shoot(N.RBG_SHOOT_RANDOM_SPHERICAL_CONE, [theta], n, lam, rot, tr, None, seed, first_id)

    @staticmethod
    def RandomSquare(lam, d, n, rot=None, tr=None, v=None, seed=None, first_id=0):
        return ARayShooter.RandomRectangle(lam, d, d, n, rot, tr, v, seed, first_id)

    @staticmethod
    def Rectangle(lam, dx, dy, nx, ny, rot=None, tr=None, v=None):
        return ARayShooter._shoot(N.RBG_SHOOT_RECTANGLE, [dx, dy, nx, ny], nx * ny, lam, rot, tr, v)

    @staticmethod
    def Square(lam, d, n, rot=None, tr=None, v=None):
        return ARayShooter.Rectangle(lam, d, d, n, n, rot, tr, v)


# ---------------------------------------------------------------------------
# scene description builder
# ---------------------------------------------------------------------------
class SceneBuilder:
    """Collects volumes, shapes, matrices, tables and materials reachable
    from a top volume into the flat arrays of rbg_scene_desc."""

    def __init__(self, top: TGeoVolume):
        self.params: List[float] = []
        self.shapes: List[N.ShapeDesc] = []
        self.shape_ids: Dict[int, int] = {}
        self.matrices: List[float] = []
        self.matrix_ids: Dict[int, int] = {}
        self.volumes: List[N.VolumeDesc] = []
        self.volume_ids: Dict[int, int] = {}
        self.volume_objs: List[TGeoVolume] = []
        self.placements: List[N.PlacementDesc] = []
        self.tables: List[N.TableDesc] = []
        self.table_ids: Dict[int, int] = {}
        self.indices: List[N.IndexDesc] = []
        self.index_ids: Dict[int, int] = {}
        self.layers: List[N.LayerDesc] = []
        self.multilayers: List[N.MultilayerDesc] = []
        self.multilayer_ids: Dict[int, int] = {}
        self.borders: List[N.BorderDesc] = []
        self.top = self.volume(top)
        # placements after all volumes exist (ids are stable)
        for vol in list(self.volume_objs):
            pass
        self._place_all()
        self._borders()

    # -- pools --------------------------------------------------------------
    def _push(self, vals):
        off = len(self.params)
        self.params.extend(float(v) for v in vals)
        return off, len(vals)

    def matrix(self, m: Optional[TGeoMatrix]) -> int:
        if m is None:
            return -1
        key = id(m)
        if key not in self.matrix_ids:
            self.matrix_ids[key] = len(self.matrices) // 12
            self.matrices.extend(float(v) for v in m.as12())
        return self.matrix_ids[key]

    def shape(self, s: TGeoShape) -> int:
        key = id(s)
        if key in self.shape_ids:
            return self.shape_ids[key]
        if isinstance(s, TGeoCompositeShape):
            left = self.shape(s.left)
            right = self.shape(s.right)
            d = N.ShapeDesc(N.SHAPE_COMPOSITE, 0, 0, s.op, left, right, self.matrix(s.left_matrix),
                            self.matrix(s.right_matrix))
        else:
            off, n = self._push(s.params())
            d = N.ShapeDesc(s.type_id, off, n, 0, -1, -1, -1, -1)
        self.shapes.append(d)
        self.shape_ids[key] = len(self.shapes) - 1
        return self.shape_ids[key]

    def table(self, t) -> int:
        if t is None:
            return -1
        key = id(t)
        if key in self.table_ids:
            return self.table_ids[key]
        if isinstance(t, TGraph):
            off, _ = self._push(list(t.x) + list(t.y))
            d = N.TableDesc(N.TABLE_1D, len(t.x), 1, off)
        elif isinstance(t, (TGraph2D, TH2)):
            xs, ys, z = t.grid()
            off, _ = self._push(list(xs) + list(ys) + list(np.asarray(z).reshape(-1)))
            d = N.TableDesc(N.TABLE_2D, len(xs), len(ys), off)
        else:
            raise TypeError(f"unsupported table {type(t).__name__}")
        self.tables.append(d)
        self.table_ids[key] = len(self.tables) - 1
        return self.table_ids[key]

    def index(self, idx: Optional[ARefractiveIndex]) -> int:
        if idx is None:
            return -1
        key = id(idx)
        if key in self.index_ids:
            return self.index_ids[key]
        ma = mb = -1
        if idx.kind == N.INDEX_MIXED:
            ma, mb = self.index(idx.a), self.index(idx.b)
        d = N.IndexDesc(idx.kind, self.table(idx.n_graph), self.table(idx.k_graph), ma, mb,
                        (C.c_double * 6)(*idx.coefficients()))
        self.indices.append(d)
        self.index_ids[key] = len(self.indices) - 1
        return self.index_ids[key]

    def multilayer(self, m: Optional[AMultilayer]) -> int:
        if m is None:
            return -1
        key = id(m)
        if key in self.multilayer_ids:
            return self.multilayer_ids[key]
        ids = [self.index(idx) for idx, _, _ in m.layers]
        off = len(self.layers)
        for (idx, th, coh), iid in zip(m.layers, ids):
            self.layers.append(N.LayerDesc(iid, int(bool(coh)), th if math.isfinite(th) else 0.0))
        md = N.MultilayerDesc(off, len(m.layers))
        if m.precalc is not None:
            kind, nl, lmin, lmax, nt, tmin, tmax = m.precalc
            md.precalc, md.lam_nbins, md.th_nbins = kind, nl, nt
            md.lam_min, md.lam_max, md.th_min, md.th_max = lmin, lmax, tmin, tmax
        self.multilayers.append(md)
        self.multilayer_ids[key] = len(self.multilayers) - 1
        return self.multilayer_ids[key]

    def volume(self, v: TGeoVolume) -> int:
        key = id(v)
        if key in self.volume_ids:
            return self.volume_ids[key]
        vid = len(self.volumes)
        self.volume_ids[key] = vid
        self.volume_objs.append(v)
        self.volumes.append(N.VolumeDesc())  # placeholder, filled below
        d = N.VolumeDesc(self.shape(v.shape), v.kind, 1.0, -1, -1, -1, -1)
        if isinstance(v, AMirror):
            d.reflectance = v.reflectance
            d.refl_table = self.table(v.reflectance_table)
        if isinstance(v, ALens):
            d.index = self.index(v.index)
        if isinstance(v, AFocalSurface):
            d.qe_lambda_table = self.table(v.qe_lambda)
            d.qe_angle_table = self.table(v.qe_angle)
        self.volumes[vid] = d
        for child, _, _, _ in v.nodes:
            self.volume(child)
        return vid

    def _place_all(self):
        for v in self.volume_objs:
            mid = self.volume_ids[id(v)]
            for child, copy_no, mat, overlap in v.nodes:
                self.placements.append(N.PlacementDesc(mid, self.volume_ids[id(child)], self.matrix(mat),
                                                       copy_no, int(overlap)))

    def _borders(self):
        for v in self.volume_objs:
            for c in getattr(v, "conditions", []):
                c2 = -1
                if c.component2 is not None:
                    if id(c.component2) not in self.volume_ids:
                        continue  # the other side is not in this scene
                    c2 = self.volume_ids[id(c.component2)]
                self.borders.append(N.BorderDesc(self.volume_ids[id(v)], c2, c.sigma,
                                                 self.multilayer(c.multilayer), int(c.lambertian)))

    def desc(self) -> N.SceneDesc:
        def arr(ctype, items):
            a = (ctype * max(1, len(items)))(*items)
            return a

        self._keep = [
            arr(N.ShapeDesc, self.shapes), arr(C.c_double, self.matrices), arr(N.VolumeDesc, self.volumes),
            arr(N.PlacementDesc, self.placements), arr(N.TableDesc, self.tables),
            arr(N.IndexDesc, self.indices), arr(N.LayerDesc, self.layers),
            arr(N.MultilayerDesc, self.multilayers), arr(N.BorderDesc, self.borders),
            arr(C.c_double, self.params),
        ]
        k = self._keep
        return N.SceneDesc(len(self.shapes), k[0], len(self.matrices) // 12, k[1], len(self.volumes), k[2],
                           len(self.placements), k[3], self.top, len(self.tables), k[4], len(self.indices), k[5],
                           len(self.layers), k[6], len(self.multilayers), k[7], len(self.borders), k[8],
                           len(self.params), k[9])


class Scene:
    """Owns a native rbg_scene handle."""

    def __init__(self, top: TGeoVolume):
        self.builder = SceneBuilder(top)
        self.desc = self.builder.desc()
        h = C.c_void_p()
        N.check(N.lib().rbg_scene_create(C.byref(self.desc), C.byref(h)), "rbg_scene_create")
        self.handle = h
        self.flat = N.FlatScene()
        N.check(N.lib().rbg_scene_flat(h, C.byref(self.flat)), "rbg_scene_flat")

    def node_names(self):
        """Physical node id -> volume name, for node histories."""
        names = []
        for i in range(self.flat.n_nodes):
            names.append(self.builder.volume_objs[self.flat.nodes[i].volume].name)
        return names

    def node_root_names(self):
        """Physical node id -> TGeoNode::GetName(), "<volume>_<copy number>"
        (TGeoVolume::AddNode names its node so; the top node is "<top>_1").

        Physical ids are the breadth-first expansion of the placements,
        children of a node in insertion order; the copy numbers are
        recovered by walking the same expansion."""
        if getattr(self, "_root_names", None) is None:
            vols = self.builder.volume_objs
            names = [vols[self.flat.nodes[0].volume].name + "_1"]
            copies = [None]
            for i in range(self.flat.n_nodes):
                nd = self.flat.nodes[i]
                kids = vols[nd.volume].nodes
                assert nd.child_count == len(kids)
                for k, (child, copy_no, _, _) in enumerate(kids):
                    cid = self.flat.children[nd.child_begin + k]
                    assert cid == len(names)
                    names.append(f"{child.name}_{copy_no}")
                    copies.append(copy_no)
            self._root_names = names
        return self._root_names

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                N.lib().rbg_scene_destroy(h)
            except Exception:
                pass
            self.handle = None


# ---------------------------------------------------------------------------
# the manager
# ---------------------------------------------------------------------------
class AOpticsManager:
    """Drop-in for ROBAST's AOpticsManager (include/AOpticsManager.h:28-103)."""

    kLens, kObs, kMirror, kFocus, kOpt, kOther, kNull = range(7)

    def __init__(self, name: str = "", title: str = ""):
        self.name, self.title = name, title
        self.top: Optional[TGeoVolume] = None
        self.limit = 100
        self.disable_fresnel = False
        self.scene: Optional[Scene] = None
        self.seed = 0x5EED5EED
        self.precision = N.PREC_FP64
        self.ray_id_offset = 0
        self.compaction = 0  # mixed tracer refill threshold, 0: the scene's tuned value
        self.ray_order = N.ORDER_SPATIAL  # mixed tracer take-up order (results do not depend on it)

    # units (include/AOpticsManager.h:59-71)
    @staticmethod
    def cm():
        return 1.0

    @staticmethod
    def m():
        return 100.0

    @staticmethod
    def km():
        return 1e5

    @staticmethod
    def mm():
        return 0.1

    @staticmethod
    def um():
        return 1e-4

    @staticmethod
    def nm():
        return 1e-7

    @staticmethod
    def inch():
        return 2.54

    @staticmethod
    def s():
        return 1.0

    @staticmethod
    def ms():
        return 1e-3

    @staticmethod
    def us():
        return 1e-6

    @staticmethod
    def ns():
        return 1e-9

    @staticmethod
    def deg():
        return math.pi / 180.0

    @staticmethod
    def rad():
        return 1.0

    def SetTopVolume(self, vol: TGeoVolume):
        self.top = vol
        self.scene = None

    def GetTopVolume(self):
        return self.top

    def CloseGeometry(self):
        if self.top is None:
            raise RuntimeError("no top volume")
        self.scene = Scene(self.top)
        return self.scene

    def SetLimit(self, n: int):
        if n > 0:
            self.limit = int(n)

    def GetLimit(self):
        return self.limit

    def DisableFresnelReflection(self, disable: bool):
        self.disable_fresnel = bool(disable)

    def SetMaxThreads(self, n):  # host threading has no role on the GPU path
        pass

    def SetMultiThread(self, flag):
        pass

    def SetNsegments(self, n):  # display only in the reference
        pass

    def IsLens(self, vol):
        return isinstance(vol, ALens)

    def IsMirror(self, vol):
        return isinstance(vol, AMirror)

    def IsFocalSurface(self, vol):
        return isinstance(vol, AFocalSurface)

    def IsObscuration(self, vol):
        return isinstance(vol, AObscuration)

    def IsOpticalComponent(self, vol):
        """An AOpticalComponent that is none of the four special kinds
        (include/AOpticsManager.h:82-90)."""
        return isinstance(vol, AOpticalComponent) and not isinstance(vol, (ALens, AMirror, AFocalSurface,
                                                                           AObscuration))

    def trace_options(self, precision=None) -> N.TraceOpts:
        o = N.TraceOpts()
        N.lib().rbg_trace_opts_default(C.byref(o))
        o.limit = self.limit
        o.disable_fresnel = int(self.disable_fresnel)
        o.seed = self.seed
        o.ray_id_offset = self.ray_id_offset
        o.precision = self.precision if precision is None else precision
        o.compaction = int(self.compaction)
        o.ray_order = int(self.ray_order)
        return o

    def _ensure_scene(self) -> Scene:
        if self.scene is None:
            self.CloseGeometry()
        return self.scene

    def TraceNonSequential(self, rays, precision=None, history: int = 0):
        """Trace an ARayArray (in place), a single ARay, or a list of ARays."""
        if isinstance(rays, ARay):
            # a single ray keeps its full history, as an ARay does
            arr = ARayArray()
            arr.Add(rays)
            cap = max(history, self.limit + 3)
            self.TraceNonSequential(arr, precision, history=cap)
            rays.status = int(arr.status[0])
            rays.npoints = int(rays.npoints + arr.npoints[0] - 1)
            rays.last_node = int(arr.last_node[0])
            m = min(int(arr.npoints[0]), cap)
            rays.points.extend(tuple(float(v) for v in arr.hist_xyzt[0, j]) for j in range(1, m))
            if m < int(arr.npoints[0]):
                rays.points.append(tuple(arr.points()[0]))
            rays.nodes.extend(int(v) for v in arr.hist_node[0, 1:m])
            rays.node_names = arr.node_names
            rays.direction = arr.directions()[0]
            return rays
        if isinstance(rays, (list, tuple)):
            arr = ARayArray()
            for r in rays:
                arr.Add(r)
            return self.TraceNonSequential(arr, precision, history)
        scene = self._ensure_scene()
        n = len(rays)
        res, keep = make_result(n, history)
        opts = self.trace_options(precision)
        rs = rays.rays_struct()
        st = N.lib().rbg_trace_host(scene.handle, C.byref(rs), C.byref(res), C.byref(opts))
        if st not in (N.RBG_OK, N.RBG_ERR_NAN, N.RBG_ERR_CAP):
            N.check(st, "rbg_trace_host")
        out = keep
        rays.x, rays.y, rays.z, rays.t = out["x"], out["y"], out["z"], out["t"]
        rays.dx, rays.dy, rays.dz = out["dx"], out["dy"], out["dz"]
        rays.status, rays.npoints, rays.last_node = out["status"], out["npoints"], out["last_node"]
        if history:
            rays.hist_xyzt, rays.hist_node = out["hist_xyzt"], out["hist_node"]
            rays.node_names = scene.node_root_names()
        rays.trace_status = st
        return rays


def make_result(n: int, history: int = 0):
    """Host result buffers + the ctypes rbg_result pointing at them."""
    keep = {k: np.zeros(n) for k in ("x", "y", "z", "t", "dx", "dy", "dz")}
    keep["status"] = np.zeros(n, dtype=np.uint8)
    keep["npoints"] = np.zeros(n, dtype=np.int32)
    keep["last_node"] = np.zeros(n, dtype=np.int32)
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int32)
    res = N.Result()
    res.status = keep["status"].ctypes.data_as(C.POINTER(C.c_uint8))
    res.npoints = keep["npoints"].ctypes.data_as(ip)
    res.last_node = keep["last_node"].ctypes.data_as(ip)
    for k in ("x", "y", "z", "t", "dx", "dy", "dz"):
        setattr(res, k, keep[k].ctypes.data_as(dp))
    res.hist_cap = int(history)
    if history:
        keep["hist_xyzt"] = np.zeros((n, history, 4))
        keep["hist_node"] = np.full((n, history), -3, dtype=np.int32)
        res.hist_xyzt = keep["hist_xyzt"].ctypes.data_as(dp)
        res.hist_node = keep["hist_node"].ctypes.data_as(ip)
    return res, keep
