"""Thin films beyond the per-ray coherent stack: AMultilayer::IncoherentTMM
(src/AMultilayer.cxx:555-731) pinned to the tmm.py values the reference's
own test holds (tutorials/unittest_robast.py:712-780), the precalculated
(lambda, theta) tables of PreCalculateCoherentTMM / PreCalculateIncoherentTMM
(include/AMultilayer.h:243-282) against direct evaluation
(unittest_robast.py:698-710), and, on the GPU, the batched FP64 evaluation
rbg_multilayer_rt and a trace through a tabulated coating against the
oracle."""
import cmath
import ctypes as C
import math

import numpy as np
import pytest

import oracle_ref as O
import robast_gb300 as R
from robast_gb300 import _native as N
from helpers import MaterialScene, deg, nm

# tmm.inc_tmm values quoted by the reference's test
RS, TS = 0.3776110935131179, 1.2856977234844612e-05
RP, TP = 0.03199545463016445, 2.0900281396463212e-05


def _inc_scene():
    n0 = R.ARefractiveIndex(1.0, 0.1)
    n1 = R.ARefractiveIndex(2.0, 0.2)
    n2 = R.ARefractiveIndex(3.0, 0.004)
    n3 = R.ARefractiveIndex(4.0, 0.2)
    d1, d2 = 100, 1000
    ml = R.AMultilayer(n0, n3)
    for idx, d, coh in ((n1, d1, True), (n2, d2, False), (n1, d1, True), (n2, d1, True), (n3, d1, True),
                        (n1, d2, False), (n3, d1, True), (n1, d1, True)):
        ml.InsertLayer(idx, d, coh)
    ms = MaterialScene(indices=[n0, n1, n2, n3], multilayers=[ml])
    # th_0 = arcsin(n00 / n0 sin(th00)) with n00 = 1, th00 = pi/3, n0 = 1 + 0.1j
    th0 = cmath.asin(1.0 / complex(1.0, 0.1) * math.sin(math.pi / 3))
    return ms, ms.ml_id[id(ml)], th0


def test_incoherent_tmm_golden_oracle():
    ms, ml, th0 = _inc_scene()
    r, t = O.tmm_c(ms.scene, ml, 0, th0, 400.0, incoherent=True)
    assert r == pytest.approx(RS, abs=5e-8) and t == pytest.approx(TS, rel=1e-6)
    r, t = O.tmm_c(ms.scene, ml, 1, th0, 400.0, incoherent=True)
    assert r == pytest.approx(RP, abs=5e-8) and t == pytest.approx(TP, rel=1e-6)


def test_incoherent_equals_coherent_when_all_coherent_oracle():
    # with every inner layer coherent, IncoherentTMM has one stack: the
    # coherent result (tmm.py's own consistency check)
    a, b = R.ARefractiveIndex(1.0), R.ARefractiveIndex(1.5, 0.01)
    h, l = R.ARefractiveIndex(2.4, 0.001), R.ARefractiveIndex(1.46)
    ml = R.AMultilayer(a, b)
    for _ in range(4):
        ml.InsertLayer(h, 47 * nm)
        ml.InsertLayer(l, 77 * nm)
    ms = MaterialScene(indices=[a, b, h, l], multilayers=[ml])
    for th in (0.0, 0.4, 1.1):
        for pol in (0, 1):
            rc, tc = O.tmm_c(ms.scene, ms.ml_id[id(ml)], pol, th, 450 * nm)
            ri, ti = O.tmm_c(ms.scene, ms.ml_id[id(ml)], pol, th, 450 * nm, incoherent=True)
            assert ri == pytest.approx(rc, abs=1e-12) and ti == pytest.approx(tc, abs=1e-12)


def _basic_multi(precalc=None):
    med1, med2 = R.ARefractiveIndex(1.), R.ARefractiveIndex(2., 4.)
    med3, med4 = R.ARefractiveIndex(3., .3), R.ARefractiveIndex(1., .1)
    multi = R.AMultilayer(med1, med4)
    multi.InsertLayer(med2, 2)
    multi.InsertLayer(med3, 3)
    if precalc:
        precalc(multi)
    ms = MaterialScene(indices=[med1, med2, med3, med4], multilayers=[multi])
    return ms, ms.ml_id[id(multi)]


def test_precalculated_table_matches_direct_oracle():
    ms0, ml0 = _basic_multi()
    ms1, ml1 = _basic_multi(lambda m: m.PreCalculateCoherentTMM(801, 199.5, 1000.5, 90, -0.5 * deg, 89.5 * deg))
    r0, t0 = O.tmm(ms0.scene, ml0, "mixed", 45 * deg, 600)
    r1, t1 = O.tmm(ms1.scene, ml1, "mixed", 45 * deg, 600)
    assert r1 == pytest.approx(r0, abs=5e-8) and t1 == pytest.approx(t0, abs=5e-8)
    # between bin centres the table interpolates; outside its range it is 0
    r2, _ = O.tmm(ms1.scene, ml1, "mixed", 45.3 * deg, 600.4)
    rd, _ = O.tmm(ms0.scene, ml0, "mixed", 45.3 * deg, 600.4)
    assert r2 == pytest.approx(rd, abs=1e-3)
    assert O.tmm(ms1.scene, ml1, "mixed", 45 * deg, 1000.6) == (0.0, 0.0)


# ---- GPU --------------------------------------------------------------------
def _rt(ms, ml, mode, pol, th, lam):
    import torch

    dev = "cuda:0"
    th = np.atleast_1d(np.asarray(th, dtype=complex))
    lam = np.broadcast_to(np.asarray(lam, dtype=float), th.shape).copy()
    t_re = torch.tensor(th.real, device=dev)
    t_im = torch.tensor(th.imag, device=dev)
    l = torch.tensor(lam, device=dev)
    R_, T_ = torch.empty_like(l), torch.empty_like(l)
    st = torch.cuda.current_stream().cuda_stream
    N.check(N.lib().rbg_multilayer_rt(ms.scene.handle, ml, mode, pol, len(l), t_re.data_ptr(), t_im.data_ptr(),
                                      l.data_ptr(), R_.data_ptr(), T_.data_ptr(), C.c_void_p(st)), "multilayer_rt")
    return R_.cpu().numpy(), T_.cpu().numpy()


@pytest.mark.gpu
def test_gpu_incoherent_and_coherent_golden():
    ms, ml, th0 = _inc_scene()
    r, t = _rt(ms, ml, 1, 0, th0, 400.0)
    assert r[0] == pytest.approx(RS, abs=5e-8) and t[0] == pytest.approx(TS, rel=1e-6)
    r, t = _rt(ms, ml, 1, 1, th0, 400.0)
    assert r[0] == pytest.approx(RP, abs=5e-8) and t[0] == pytest.approx(TP, rel=1e-6)
    msb, mlb = _basic_multi()
    r, t = _rt(msb, mlb, 0, 0, 0.1, 100.0)
    assert r[0] == pytest.approx(0.37273208839139516, abs=5e-8) and t[0] == pytest.approx(0.22604491247079261,
                                                                                           abs=5e-8)


@pytest.mark.gpu
def test_gpu_batches_match_oracle():
    ms, ml, _ = _inc_scene()
    g = np.random.default_rng(2)
    th = g.uniform(0, 1.3, 64) + 0j
    lam = g.uniform(300, 700, 64)
    for mode, inc in ((0, False), (1, True)):
        for pol in (0, 1):
            r, t = _rt(ms, ml, mode, pol, th, lam)
            for k in range(0, 64, 7):
                ro, to = O.tmm_c(ms.scene, ml, pol, th[k], lam[k], incoherent=inc)
                assert r[k] == pytest.approx(ro, rel=1e-9, abs=1e-13) and t[k] == pytest.approx(to, rel=1e-9,
                                                                                                 abs=1e-13)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["coherent", "incoherent"])
def test_gpu_table_matches_oracle(kind):
    def pre(m):
        f = m.PreCalculateCoherentTMM if kind == "coherent" else m.PreCalculateIncoherentTMM
        f(81, 199.5, 1000.5, 30, -0.5 * deg, 89.5 * deg)

    ms, ml = _basic_multi(pre)
    g = np.random.default_rng(4)
    th = g.uniform(0, 1.5, 200)
    lam = g.uniform(150, 1100, 200)  # some outside the table: 0
    r, t = _rt(ms, ml, 2, 2, th, lam)
    for k in range(0, 200, 9):
        ro, to = O.tmm(ms.scene, ml, "mixed", th[k], lam[k])
        assert r[k] == pytest.approx(ro, rel=1e-9, abs=1e-12) and t[k] == pytest.approx(to, rel=1e-9, abs=1e-12)
    assert (r[lam > 1000.5] == 0).all()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [N.PREC_FP64, N.PREC_MIXED])
def test_trace_through_tabulated_coating(prec):
    """Rays onto a mirror whose border condition is a precalculated stack:
    the per-ray reflectance is the table's, identically on the GPU and in
    the oracle (same Philox draws)."""
    import torch

    from robast_gb300 import device
    from helpers import make_the_world

    man = make_the_world()
    world = man.GetTopVolume()
    a, b = R.ARefractiveIndex(1.0), R.ARefractiveIndex(1.52)
    h, l = R.ARefractiveIndex(2.4, 0.002), R.ARefractiveIndex(1.46)
    ml = R.AMultilayer(a, b)
    for _ in range(5):
        ml.InsertLayer(h, 450 * nm / 4 / 2.4)
        ml.InsertLayer(l, 450 * nm / 4 / 1.46)
    ml.PreCalculateIncoherentTMM(60, 300 * nm, 700 * nm, 45, 0.0, 90 * deg)
    mirror = R.AMirror("coated", R.TGeoBBox("cb", 50, 50, 0.01))
    world.AddNode(mirror, 1)
    cond = R.ABorderSurfaceCondition(world, mirror)
    cond.SetMultilayer(ml)
    man.CloseGeometry()
    n = 20000
    g = np.random.default_rng(8)
    th = g.uniform(0, 80 * deg, n)
    d = np.stack([np.sin(th), np.zeros(n), -np.cos(th)], axis=1)
    batch = {"x": g.uniform(-10, 10, n) - 5 * d[:, 0] / np.cos(th), "y": g.uniform(-10, 10, n), "z": np.full(n, 5.0),
             "dx": d[:, 0], "dy": d[:, 1], "dz": d[:, 2], "lam": g.uniform(320 * nm, 680 * nm, n)}
    res, st = device.trace(man, device.to_device(batch, "cuda:0"), precision=prec)
    torch.cuda.synchronize()
    assert st == N.RBG_OK
    got = {k: v.cpu().numpy() for k, v in res.items()}
    arr = R.ARayArray.from_arrays(batch["x"], batch["y"], batch["z"], batch["dx"], batch["dy"], batch["dz"],
                                  batch["lam"])
    ost, ref = O.trace(man, arr, threads=8)
    assert ost == 0
    agree = (got["status"] == ref["status"]).mean()
    assert agree >= 0.999
    absorbed = (ref["status"] == N.RBG_ABSORB).mean()
    assert 0.01 < absorbed < 0.99
