"""AGeoWinstonCone2D and AGeoBezierPcon / AGeoBezierPgon.

The 2D cone is a compound parabolic trough: for rays in its x-z plane it
is an ideal concentrator with cutoff asin(r2/r1) -- a closed-form
known-answer test of the oracle's restatement of
src/AGeoWinstonCone2D.cxx, then GPU parity with the oracle.  The Bezier
shapes are polycones/polygons whose sections sample the reference's
Bezier curve (src/AGeoBezierPcon.cxx:35-80): the sections against the
closed form, then a Bezier funnel traced on the GPU against the oracle."""
import math

import numpy as np
import pytest

import oracle_ref
import robast_gb300 as R
from robast_gb300 import _native as N
from helpers import cm, deg, nm

R1, R2, DY = 2.5, 1.25, 3.0


def _trough_scene():
    man = R.AOpticsManager("manager", "trough")
    world = R.AOpticalComponent("world", R.TGeoBBox("worldbox", 50 * cm, 50 * cm, 50 * cm))
    man.SetTopVolume(world)
    cone = R.AGeoWinstonCone2D("trough", R1, R2, DY)
    dz = cone.GetDZ()
    block = R.AMirror("block", R.TGeoBBox("blockbox", R1 + 0.5, DY + 0.5, dz))
    block.SetReflectance(1.0)
    block.AddNode(R.AOpticalComponent("interior", cone), 1)
    world.AddNode(block, 1)
    sensor = R.AFocalSurface("sensor", R.TGeoBBox("sensorbox", R1 + 0.5, DY + 0.5, 0.05))
    world.AddNode(sensor, 1, R.TGeoTranslation(0, 0, -dz - 0.06))
    man.CloseGeometry()
    return man, dz


def _trough_rays(alpha, n, dz, seed=1):
    g = np.random.default_rng(seed)
    x = g.uniform(-0.95 * R1, 0.95 * R1, n)
    y = g.uniform(-0.9 * DY, 0.9 * DY, n)
    s = 1.0 / math.cos(alpha)
    d = np.array([math.sin(alpha), 0.0, -math.cos(alpha)])
    z0 = dz + 1.0
    return {"x": x - s * d[0], "y": y, "z": np.full(n, z0), "dx": np.full(n, d[0]), "dy": np.zeros(n),
            "dz": np.full(n, d[2]), "lam": np.full(n, 400 * nm)}


def _arr(b):
    return R.ARayArray.from_arrays(b["x"], b["y"], b["z"], b["dx"], b["dy"], b["dz"], b["lam"])


def test_trough_acceptance_cutoff_oracle():
    man, dz = _trough_scene()
    cut = math.asin(R2 / R1)
    for frac, expect in ((0.5, 1.0), (0.9, 1.0), (1.1, 0.0), (1.5, 0.0)):
        st, out = oracle_ref.trace(man, _arr(_trough_rays(frac * cut, 2000, dz)), threads=8)
        assert st == 0
        focused = (out["status"] == N.RBG_FOCUS).mean()
        assert abs(focused - expect) < 0.02, (frac, focused)


def test_trough_shape_queries_oracle():
    man, dz = _trough_scene()
    sc = man._ensure_scene()
    sid = [i for i in range(sc.flat.n_shapes) if sc.flat.shapes[i].type == N.SHAPE_WINSTON_2D][0]
    L = oracle_ref.lib()
    import ctypes as C

    def v(*a):
        return (C.c_double * 3)(*a)

    assert L.orc_shape_contains(C.byref(sc.flat), sid, v(0, 0, 0)) == 1
    assert L.orc_shape_contains(C.byref(sc.flat), sid, v(0, DY + 0.01, 0)) == 0
    assert L.orc_shape_contains(C.byref(sc.flat), sid, v(R1 * 0.99, 0, dz * 0.999)) == 1
    assert L.orc_shape_contains(C.byref(sc.flat), sid, v(R2 * 1.01, 0, -dz * 0.999)) == 0
    # straight down through the entrance: enter at z = dz, leave at z = -dz
    assert L.orc_shape_dist_out(C.byref(sc.flat), sid, v(0.1, 0.2, dz + 2), v(0, 0, -1)) == pytest.approx(2.0)
    assert L.orc_shape_dist_in(C.byref(sc.flat), sid, v(0.1, 0.2, 0), v(0, 0, -1)) == pytest.approx(dz)
    # along +y the trough ends at |y| = DY
    assert L.orc_shape_dist_in(C.byref(sc.flat), sid, v(0, 0, 0), v(0, 1, 0)) == pytest.approx(DY)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [N.PREC_FP64, N.PREC_MIXED])
def test_trough_gpu_parity(prec):
    import torch

    from robast_gb300 import device

    man, dz = _trough_scene()
    cut = math.asin(R2 / R1)
    parts = [_trough_rays(a * cut, 3000, dz, seed=i) for i, a in enumerate((0.3, 0.8, 0.95, 1.05, 1.3))]
    b = {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}
    res, st = device.trace(man, device.to_device(b, "cuda:0"), precision=prec)
    torch.cuda.synchronize()
    assert st == N.RBG_OK
    got = {k: v.cpu().numpy() for k, v in res.items()}
    ost, ref = oracle_ref.trace(man, _arr(b), threads=8)
    assert ost == 0
    same = (got["status"] == ref["status"]) & (got["npoints"] == ref["npoints"]) & (got["last_node"] == ref["last_node"])
    assert same.mean() >= 0.999
    for k in ("x", "y", "z"):
        np.testing.assert_allclose(got[k][same], ref[k][same], rtol=1e-6, atol=1e-6)
    assert (got["npoints"] > 3).any()  # multiple wall bounces happen


# ---- Bezier polycones -------------------------------------------------------
def _bezier_ref(t, n, p1, p2, r1, r2, dz):
    if n == 0:
        bx, by = t, t
    elif n == 1:
        bx = 2 * (1 - t) * t * p1[0] + t * t
        by = 2 * (1 - t) * t * p1[1] + t * t
    else:
        bx = 3 * (1 - t) ** 2 * t * p1[0] + 3 * (1 - t) * t * t * p2[0] + t ** 3
        by = 3 * (1 - t) ** 2 * t * p1[1] + 3 * (1 - t) * t * t * p2[1] + t ** 3
    return r2 + bx * (r1 - r2), -dz + by * 2 * dz


@pytest.mark.parametrize("ctrl", [(), ((0.8, 0.2),), ((0.1, 0.6), (0.9, 0.3))])
@pytest.mark.parametrize("cls", ["pcon", "pgon"])
def test_bezier_sections(ctrl, cls):
    r1, r2, dz, nz = 4.0, 1.5, 3.0, 9
    s = R.AGeoBezierPcon("b", 0, 360, nz, r1, r2, dz) if cls == "pcon" else \
        R.AGeoBezierPgon("b", 0, 360, 6, nz, r1, r2, dz)
    if ctrl:
        s.SetControlPoints(*[c for p in ctrl for c in p])
    else:
        s.SetSections()
    p1 = ctrl[0] if ctrl else (0, 0)
    p2 = ctrl[1] if len(ctrl) > 1 else (0, 0)
    for i in range(nz):
        r, z = _bezier_ref(i / (nz - 1), len(ctrl), p1, p2, r1, r2, dz)
        assert s.rmax[i] == pytest.approx(r, rel=1e-14, abs=1e-14)
        assert s.z[i] == pytest.approx(z, rel=1e-14, abs=1e-14)
        assert s.rmin[i] == 0


def _funnel_scene():
    man = R.AOpticsManager("manager", "funnel")
    world = R.AOpticalComponent("world", R.TGeoBBox("worldbox", 50 * cm, 50 * cm, 50 * cm))
    man.SetTopVolume(world)
    outer = R.TGeoBBox("outerbox", 6, 6, 3)
    block = R.AMirror("block", outer)
    block.SetReflectance(0.9)
    hole = R.AGeoBezierPgon("hole", 0, 360, 6, 12, 4.0, 1.5, 3.0)
    hole.SetControlPoints(0.3, 0.7, 0.8, 0.9)
    block.AddNode(R.AOpticalComponent("holevol", hole), 1)
    world.AddNode(block, 1)
    world.AddNode(R.AFocalSurface("sensor", R.TGeoBBox("sb", 6, 6, 0.05)), 1, R.TGeoTranslation(0, 0, -3.06))
    man.CloseGeometry()
    return man


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [N.PREC_FP64, N.PREC_MIXED])
def test_bezier_funnel_gpu_parity(prec):
    import torch

    from robast_gb300 import device

    man = _funnel_scene()
    g = np.random.default_rng(3)
    n = 20000
    th = np.radians(g.uniform(0, 35, n))
    ph = g.uniform(0, 2 * np.pi, n)
    d = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), -np.cos(th)], axis=1)
    x0, y0 = g.uniform(-3.4, 3.4, n), g.uniform(-3.4, 3.4, n)
    s = 2.0 / np.cos(th)
    b = {"x": x0 - s * d[:, 0], "y": y0 - s * d[:, 1], "z": np.full(n, 5.0), "dx": d[:, 0], "dy": d[:, 1],
         "dz": d[:, 2], "lam": np.full(n, 400 * nm)}
    res, st = device.trace(man, device.to_device(b, "cuda:0"), precision=prec)
    torch.cuda.synchronize()
    assert st == N.RBG_OK
    got = {k: v.cpu().numpy() for k, v in res.items()}
    ost, ref = oracle_ref.trace(man, _arr(b), threads=8)
    assert ost == 0
    same = (got["status"] == ref["status"]) & (got["npoints"] == ref["npoints"])
    assert same.mean() >= 0.999
    for k in ("x", "y", "z"):
        np.testing.assert_allclose(got[k][same], ref[k][same], rtol=1e-6, atol=1e-6)
    assert (got["status"] == N.RBG_FOCUS).mean() > 0.2
