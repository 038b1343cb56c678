"""Known-answer tests that pin the CPU oracle to the reference's own golden
values (tutorials/unittest_robast.py) and to published vectors."""
import ctypes as C
import math

import numpy as np
import pytest

import oracle_ref as O
import robast_gb300 as R
from helpers import MaterialScene, deg, glass_catalog, make_the_world, mm, nm, m


def test_philox_known_answers():
    # Random123 kat_vectors for philox4x32-10
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def _tmm_scene():
    # tutorials/unittest_robast.py:627-641 (tmm.tests.basic_test)
    med1 = R.ARefractiveIndex(1.)
    med2 = R.ARefractiveIndex(2., 4.)
    med3 = R.ARefractiveIndex(3., .3)
    med4 = R.ARefractiveIndex(1., .1)
    multi = R.AMultilayer(med1, med4)
    multi.InsertLayer(med2, 2)
    multi.InsertLayer(med3, 3)
    ms = MaterialScene(indices=[med1, med2, med3, med4], multilayers=[multi])
    return ms, ms.ml_id[id(multi)]


def test_tmm_golden():
    ms, ml = _tmm_scene()
    rs, rp = 0.37273208839139516, 0.37016110373044969
    ts, tp = 0.22604491247079261, 0.22824374314132009
    R_, T_ = O.tmm(ms.scene, ml, 0, 0.1, 100.0)
    assert R_ == pytest.approx(rs, abs=5e-8) and T_ == pytest.approx(ts, abs=5e-8)
    R_, T_ = O.tmm(ms.scene, ml, 1, 0.1, 100.0)
    assert R_ == pytest.approx(rp, abs=5e-8) and T_ == pytest.approx(tp, abs=5e-8)
    R_, T_ = O.tmm(ms.scene, ml, "mixed", 0.1, 100.0)
    assert R_ == pytest.approx((rs + rp) / 2, abs=5e-8) and T_ == pytest.approx((ts + tp) / 2, abs=5e-8)


def test_tmm_reversed_stack_consistent():
    # energy conservation for a lossless stack: R + T = 1
    a, b = R.ARefractiveIndex(1.0), R.ARefractiveIndex(1.52)
    h, l = R.ARefractiveIndex(2.4), R.ARefractiveIndex(1.46)
    ml = R.AMultilayer(a, b)
    for i in range(10):
        ml.InsertLayer(h, 450 * nm / 4 / 2.4)
        ml.InsertLayer(l, 450 * nm / 4 / 1.46)
    ms = MaterialScene(indices=[a, b, h, l], multilayers=[ml])
    for th in (0.0, 0.3, 0.9):
        for lam in (350 * nm, 450 * nm, 600 * nm):
            for pol in (0, 1):
                R_, T_ = O.tmm(ms.scene, ms.ml_id[id(ml)], pol, th, lam)
                assert R_ + T_ == pytest.approx(1.0, abs=1e-10)
    # quarter-wave stack: high reflectance at the centre wavelength
    R_, _ = O.tmm(ms.scene, ms.ml_id[id(ml)], "mixed", 0.0, 450 * nm)
    assert R_ > 0.999


NBK7 = (1.03961212, 0.231792344, 1.01046945, 0.00600069867, 0.0200179144, 103.560653)
NBK7_TABLE = ((2325.4, 1.489210), (1970.1, 1.494950), (1529.6, 1.500910), (1060.0, 1.506690),
              (1014.0, 1.507310), (852.1, 1.509800), (706.5, 1.512890), (656.3, 1.514320),
              (643.8, 1.514720), (632.8, 1.515090), (589.3, 1.516730), (587.6, 1.516800),
              (546.1, 1.518720), (486.1, 1.522380), (480.0, 1.522830), (435.8, 1.526680),
              (404.7, 1.530240), (365.0, 1.536270), (334.1, 1.542720), (312.6, 1.548620))


def test_sellmeier_nbk7():
    # tutorials/unittest_robast.py:530-561
    s = R.ASellmeierFormula(*NBK7)
    ms = MaterialScene(indices=[s])
    i = ms.index_id[id(s)]
    for wl, n in ((312.6, 1.548620), (589.3, 1.516730), (1014.0, 1.507310), (2325.4, 1.489210)):
        v = O.lib().orc_refractive_index(C.byref(ms.scene.flat), i, wl * nm)
        assert round(abs(v - n), 4) == 0
    for wl, n in NBK7_TABLE:
        assert abs(O.lib().orc_refractive_index(C.byref(ms.scene.flat), i, wl * nm) - n) < 1e-4
    assert round(abs(s.GetAbbeNumber() - 64.17), 1) == 0
    # a scaled formula must miss the table (the reference checks this too)
    bad = R.ASellmeierFormula(*[v * 0.95 for v in NBK7])
    assert abs(bad.GetRefractiveIndex(589.3 * nm) - 1.516730) > 1e-3


def test_glass_catalog_nbk7():
    # tutorials/unittest_robast.py:524-528
    g = glass_catalog().GetRefractiveIndex("N-BK7")
    ms = MaterialScene(indices=[g])
    i = ms.index_id[id(g)]
    nD = O.lib().orc_refractive_index(C.byref(ms.scene.flat), i, 589.3 * nm)
    assert round(nD / 1.51680 - 1.0, 4) == 0
    k = O.lib().orc_extinction(C.byref(ms.scene.flat), i, 2325 * nm)
    assert round(k - 4.2911e-6, 9) == 0
    assert glass_catalog().GetRefractiveIndex("LITHOSIL-Q") is not None


def test_refractive_index_tgraph():
    # tutorials/unittest_robast.py:415-426
    g = R.TGraph()
    g.SetPoint(0, 400 * nm, 1.6)
    g.SetPoint(1, 500 * nm, 1.5)
    idx = R.ARefractiveIndex()
    idx.SetRefractiveIndex(g)
    ms = MaterialScene(indices=[idx])
    v = O.lib().orc_refractive_index(C.byref(ms.scene.flat), ms.index_id[id(idx)], 450 * nm)
    assert v == pytest.approx(1.55, abs=1e-15)


def test_mixed_refractive_index():
    # tutorials/unittest_robast.py:612-625
    a, b = R.ARefractiveIndex(1., 1.), R.ARefractiveIndex(2., 2.)
    mix = R.AMixedRefractiveIndex(a, b, 3, 7)
    ms = MaterialScene(indices=[mix])
    i = ms.index_id[id(mix)]
    assert O.lib().orc_refractive_index(C.byref(ms.scene.flat), i, 100 * nm) == pytest.approx(0.3 + 1.4)
    assert O.lib().orc_extinction(C.byref(ms.scene.flat), i, 100 * nm) == pytest.approx(0.3 + 1.4)


def test_mirror_reflectance_tables():
    # tutorials/unittest_robast.py:202-205, 223-231
    g = R.TGraph()
    g.SetPoint(0, 300 * nm, 0.)
    g.SetPoint(1, 500 * nm, .5)
    m1 = R.AMirror("m1", R.TGeoBBox("b1", 1, 1, 1))
    m1.SetReflectance(g)
    g2 = R.TGraph2D()
    g2.SetPoint(0, 300 * nm, 0 * deg, 0.0)
    g2.SetPoint(1, 300 * nm, 90 * deg, 0.3)
    g2.SetPoint(2, 500 * nm, 0 * deg, 0.7)
    g2.SetPoint(3, 500 * nm, 90 * deg, 1.0)
    m2 = R.AMirror("m2", R.TGeoBBox("b2", 1, 1, 1))
    m2.SetReflectance(g2)
    ms = MaterialScene(mirrors=[m1, m2])
    f = C.byref(ms.scene.flat)
    assert O.lib().orc_mirror_reflectance(f, ms.volume_id[id(m1)], 400 * nm, 0) == pytest.approx(0.25, abs=1e-6)
    assert O.lib().orc_mirror_reflectance(f, ms.volume_id[id(m2)], 400 * nm, 45 * deg) == pytest.approx(0.5, abs=1e-3)
    assert m1.GetReflectance(400 * nm, 0) == pytest.approx(0.25, abs=1e-6)


def snell_scene():
    # tutorials/unittest_robast.py:428-468
    man = make_the_world()
    man.DisableFresnelReflection(True)
    lens = R.ALens("lens", R.TGeoBBox("lensbox", 0.5 * m, 0.5 * m, 1 * mm))
    lens.SetRefractiveIndex(R.ARefractiveIndex(1.5))
    man.GetTopVolume().AddNode(lens, 1)
    focal = R.AFocalSurface("focal", R.TGeoBBox("focalbox", 0.5 * m, 0.5 * m, 0.1 * mm))
    lens.AddNode(focal, 1)
    man.CloseGeometry()
    th = 30 * deg
    rays = R.ARayArray()
    rays.Add(R.ARay(0, 400 * nm, 0 * m, 0 * m, 2 * mm, 0, math.sin(th), 0, -math.cos(th)))
    return man, rays


def test_snells_law():
    man, rays = snell_scene()
    st, out = O.trace(man, rays)
    assert st == 0
    assert round(out["dx"][0] - math.sin(30 * deg) / 1.5, 7) == 0
    assert round(out["dy"][0], 7) == 0
    assert out["status"][0] == R.ARay.kFocus


def limit_scene():
    # tutorials/unittest_robast.py:390-413
    man = make_the_world(limit=1000)
    mirror = R.AMirror("mirror", R.TGeoSphere("mirrorsphere", 0.1 * m, 0.2 * m))
    man.GetTopVolume().AddNode(mirror, 1)
    man.CloseGeometry()
    rays = R.ARayArray()
    rays.Add(R.ARay(0, 400 * nm, 0, 0, 0, 0, 0, 0, -1))
    return man, rays


def test_limit_for_suspended():
    man, rays = limit_scene()
    st, out = O.trace(man, rays)
    assert out["npoints"][0] == 1000
    assert out["status"][0] == R.ARay.kSuspend


def test_d80_uniform_radial():
    # tutorials/unittest_robast.py:590-610: points at radius r0*U(0,1) in a
    # uniform direction -> 80% containment at 0.8 r0, centre (x0, y0)
    rng = np.random.default_rng(590)
    N = 2_000_000
    x0, y0, r0 = 1.0, -1.0, 2.0
    phi = rng.uniform(0, 2 * np.pi, N)
    s = rng.uniform(0, 1, N)
    x = r0 * np.cos(phi) * s + x0
    y = r0 * np.sin(phi) * s + y0
    h, _, _ = np.histogram2d(x, y, bins=[500, 500], range=[[-3, 3], [-3, 3]])
    r, cx, cy = O.containment_radius(h, -3, 3, -3, 3, 0.8)
    tol = 0.015
    assert abs(cx / x0 - 1.) <= tol
    assert abs(cy / y0 - 1.) <= tol
    assert abs(r / r0 - 0.8) / 0.8 <= tol


def test_python_tgraph_eval_matches_oracle():
    g = R.TGraph(x=[3.0, 1.0, 2.0, 5.0], y=[30.0, 10.0, 25.0, 40.0])
    idx = R.ARefractiveIndex()
    idx.SetRefractiveIndex(g)
    ms = MaterialScene(indices=[idx])
    for x in (0.0, 1.0, 1.5, 2.0, 2.7, 4.9, 7.0):
        assert O.lib().orc_refractive_index(C.byref(ms.scene.flat), ms.index_id[id(idx)], x) == \
            pytest.approx(g.Eval(x), abs=1e-12)
