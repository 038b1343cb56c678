"""AMultilayer's own evaluation calls (CoherentTMM / CoherentTMMS / P /
Mixed, IncoherentTMM / S / P / Mixed, the vector forms, `reverse` and the
precalculated tables), restating the reference's tests
tutorials/unittest_robast.py:627-780 through this package's public API.
The calls run on the GPU (rbg_multilayer_rt); the CPU test checks the
one-mirror scene they evaluate against tmm.py's values through the oracle."""
import cmath
import ctypes
import math

import numpy as np
import pytest

import oracle_ref as O
import robast_gb300 as R

deg = math.pi / 180
RS, RP = 0.37273208839139516, 0.37016110373044969
TS, TP = 0.22604491247079261, 0.22824374314132009
# tmm.inc_tmm values quoted by the reference's incoherent test
IRS, ITS = 0.3776110935131179, 1.2856977234844612e-05
IRP, ITP = 0.03199545463016445, 2.0900281396463212e-05


def _basic():
    med1, med2 = R.ARefractiveIndex(1.), R.ARefractiveIndex(2., 4.)
    med3, med4 = R.ARefractiveIndex(3., .3), R.ARefractiveIndex(1., .1)
    multi = R.AMultilayer(med1, med4)
    multi.InsertLayer(med2, 2)
    multi.InsertLayer(med3, 3)
    reverse = R.AMultilayer(med4, med1)
    reverse.InsertLayer(med3, 3)
    reverse.InsertLayer(med2, 2)
    return multi, reverse


def _incoherent():
    n0 = R.ARefractiveIndex(1.0, 0.1)
    n1 = R.ARefractiveIndex(2.0, 0.2)
    n2 = R.ARefractiveIndex(3.0, 0.004)
    n3 = R.ARefractiveIndex(4.0, 0.2)
    d1, d2 = 100, 1000
    ml = R.AMultilayer(n0, n3)
    for idx, d, coh in ((n1, d1, True), (n2, d2, False), (n1, d1, True), (n2, d1, True), (n3, d1, True),
                        (n1, d2, False), (n3, d1, True), (n1, d1, True)):
        ml.InsertLayer(idx, d, coh)
    th0 = cmath.asin(1.0 / complex(1.0, 0.1) * math.sin(math.pi / 3))
    return ml, th0


def test_evaluation_scene_restates_the_stack_oracle():
    multi, reverse = _basic()
    for ml, rev in ((multi, False), (reverse, True)):
        scene, mid = ml._scene(rev)
        r, t = O.tmm_c(scene, mid, 0, 0.1, 100.0)
        assert r == pytest.approx(RS, abs=1e-12) and t == pytest.approx(TS, abs=1e-12)
        r, t = O.tmm_c(scene, mid, 1, 0.1, 100.0)
        assert r == pytest.approx(RP, abs=1e-12) and t == pytest.approx(TP, abs=1e-12)
    # a changed thickness rebuilds the scene
    s0 = multi._scene()[0]
    multi.ChangeThickness(1, 2.5)
    assert multi._scene()[0] is not s0
    ml, th0 = _incoherent()
    scene, mid = ml._scene()
    r, t = O.tmm_c(scene, mid, 0, th0, 400.0, incoherent=True)
    assert r == pytest.approx(IRS, abs=5e-8) and t == pytest.approx(ITS, rel=1e-6)


@pytest.mark.gpu
def test_coherent_tmm_api():
    multi, reverse = _basic()
    r, t = ctypes.c_double(), ctypes.c_double()
    multi.CoherentTMM(R.AMultilayer.kS, 0.1, 100, r, t)
    assert r.value == pytest.approx(RS, abs=1e-7) and t.value == pytest.approx(TS, abs=1e-7)
    multi.CoherentTMM(R.AMultilayer.kP, 0.1, 100, r, t)
    assert r.value == pytest.approx(RP, abs=1e-7) and t.value == pytest.approx(TP, abs=1e-7)
    assert multi.CoherentTMMS(0.1, 100) == pytest.approx((RS, TS), abs=1e-7)
    assert multi.CoherentTMMP(0.1, 100) == pytest.approx((RP, TP), abs=1e-7)
    multi.CoherentTMMMixed(0.1, 100, r, t)
    assert r.value == pytest.approx((RS + RP) / 2, abs=1e-7) and t.value == pytest.approx((TS + TP) / 2, abs=1e-7)
    reverse.CoherentTMM(R.AMultilayer.kS, 0.1, 100, r, t, True)
    assert r.value == pytest.approx(RS, abs=1e-7) and t.value == pytest.approx(TS, abs=1e-7)
    reverse.CoherentTMM(R.AMultilayer.kP, 0.1, 100, r, t, True)
    assert r.value == pytest.approx(RP, abs=1e-7) and t.value == pytest.approx(TP, abs=1e-7)


@pytest.mark.gpu
def test_coherent_tmm_vector_forms_equal_scalar_calls():
    multi, _ = _basic()
    lams = list(range(300, 800, 7))
    rv, tv = [], []
    multi.CoherentTMMMixed(0.1, lams, rv, tv)
    for lam, a, b in zip(lams, rv, tv):
        assert multi.CoherentTMMMixed(0.1, lam) == pytest.approx((a, b), abs=1e-12)
    angles = [i * math.pi / 2000. for i in range(0, 500, 9)]
    ra, ta = multi.CoherentTMMMixed(angles, 100)
    for th, a, b in zip(angles, ra, ta):
        assert multi.CoherentTMMMixed(th, 100) == pytest.approx((a, b), abs=1e-12)


@pytest.mark.gpu
def test_precalculated_table_replaces_direct_evaluation():
    multi, _ = _basic()
    r0 = multi.CoherentTMMMixed(45 * deg, 600)
    multi.PreCalculateCoherentTMM(801, 199.5, 1000.5, 90, -0.5 * deg, 89.5 * deg)
    r1 = multi.CoherentTMMMixed(45 * deg, 600)
    assert r1 == pytest.approx(r0, abs=1e-7)
    # outside the table's wavelength range the table gives 0 (TH2::Interpolate)
    assert multi.CoherentTMMMixed(45 * deg, 1100) == (0.0, 0.0)


@pytest.mark.gpu
def test_incoherent_tmm_api():
    ml, th0 = _incoherent()
    r, t = ctypes.c_double(), ctypes.c_double()
    ml.IncoherentTMM(R.AMultilayer.kS, th0, 400, r, t)
    assert r.value == pytest.approx(IRS, abs=5e-8) and t.value == pytest.approx(ITS, rel=1e-6)
    ml.IncoherentTMM(R.AMultilayer.kP, th0, 400, r, t)
    assert r.value == pytest.approx(IRP, abs=5e-8) and t.value == pytest.approx(ITP, rel=1e-6)
    assert ml.IncoherentTMMS(th0, 400)[0] == pytest.approx(IRS, abs=5e-8)
    assert ml.IncoherentTMMP(th0, 400)[0] == pytest.approx(IRP, abs=5e-8)
    rm, tm = ml.IncoherentTMMMixed(th0, 400)
    assert rm == pytest.approx((IRS + IRP) / 2, abs=5e-8) and tm == pytest.approx((ITS + ITP) / 2, rel=1e-6)
