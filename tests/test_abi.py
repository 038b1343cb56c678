"""C ABI checks that need no GPU: every declared entry point is exported,
scene descriptions are validated, ray sources follow the ARayShooter laws."""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

import robast_gb300 as R
from robast_gb300 import _native as N
from helpers import make_the_world, m, nm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\**\s+\**(rbg_[a-z_0-9]+)\s*\(", src, flags=re.M))
    return sorted(names)


def test_all_declared_symbols_exported():
    names = declared_functions()
    assert "rbg_trace" in names and "rbg_scene_create" in names
    lib = N.lib()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_status_strings():
    lib = N.lib()
    assert lib.rbg_abi_version() == 2
    for s in range(9):
        assert lib.rbg_status_string(s)
    o = N.TraceOpts()
    lib.rbg_trace_opts_default(C.byref(o))
    assert o.limit == 100 and o.disable_fresnel == 0


def test_scene_flattening_tree():
    man = make_the_world()
    world = man.GetTopVolume()
    top = R.AOpticalComponent("top", R.TGeoBBox("topbox", 5 * m, 5 * m, 5 * m))
    mir = R.AMirror("mir", R.TGeoBBox("mb", 10, 10, 1))
    for i in range(20):
        top.AddNode(mir, i + 1, R.TGeoTranslation(30.0 * (i - 10), 0, 0))
    world.AddNode(top, 1, R.TGeoTranslation(0, 0, 100))
    sc = man.CloseGeometry()
    f = sc.flat
    assert f.n_nodes == 22
    assert f.nodes[0].parent == -1 and f.nodes[1].parent == 0
    assert f.nodes[1].child_count == 20 and f.nodes[1].bvh_root >= 0
    # composed transform of a grand-child
    n5 = f.nodes[2 + 5]
    assert n5.m[9] == pytest.approx(30.0 * (5 - 10)) and n5.m[11] == pytest.approx(100.0)
    assert n5.lo[2] == pytest.approx(99.0, abs=1e-3) and n5.hi[2] == pytest.approx(101.0, abs=1e-3)


def _bad_scene(mutator):
    man = make_the_world()
    man.GetTopVolume().AddNode(R.AMirror("mm", R.TGeoBBox("bb", 1, 1, 1)), 1)
    b = R.Scene.__new__(R.Scene)
    from robast_gb300.manager import SceneBuilder

    sb = SceneBuilder(man.GetTopVolume())
    mutator(sb)
    desc = sb.desc()
    h = C.c_void_p()
    return N.lib().rbg_scene_create(C.byref(desc), C.byref(h))


def test_scene_validation_errors():
    assert _bad_scene(lambda sb: None) == N.RBG_OK

    def bad_top(sb):
        sb.top = 99

    def bad_shape(sb):
        sb.volumes[0].shape = 42

    def bad_kind(sb):
        sb.volumes[0].kind = 17

    def bad_params(sb):
        sb.shapes[0].n_params = 10 ** 6

    def cycle(sb):
        sb.placements.append(N.PlacementDesc(1, 0, -1, 1, 0))

    for mut in (bad_top, bad_shape, bad_kind, bad_params):
        assert _bad_scene(mut) == N.RBG_ERR_SCENE, mut.__name__
    assert _bad_scene(cycle) == N.RBG_ERR_SCENE  # unbounded depth
    assert N.lib().rbg_scene_create(None, None) == N.RBG_ERR_ARG


def test_ageo_in_composite_rejected():
    man = make_the_world()
    a = R.AGeoAsphericDisk("asph_in_csg", 0, 0, 1, 0, 10, 0)
    b = R.TGeoBBox("box_in_csg", 5, 5, 5)
    comp = R.TGeoCompositeShape("bad_comp", op=N.OP_SUBTRACTION, left=b, right=a)
    man.GetTopVolume().AddNode(R.AMirror("mm2", comp), 1)
    with pytest.raises(N.NativeError) as e:
        man.CloseGeometry()
    assert e.value.status == N.RBG_ERR_UNSUPPORTED


def test_random_circle_law():
    n = 200_000
    arr = R.ARayShooter.RandomCircle(400 * nm, 110.0, n, None, R.TGeoTranslation(0, 0, 1600), (0, 0, -1))
    assert len(arr) == n
    r = np.hypot(arr.x, arr.y)
    assert r.max() <= 110.0
    # uniform over the disk: P(r < R/2) = 1/4
    frac = (r < 55.0).mean()
    assert abs(frac - 0.25) < 4 * math.sqrt(0.25 * 0.75 / n)
    assert np.all(arr.z == 1600) and np.all(arr.dz == -1)
    # reproducible and shard-invariant: rays 1000.. equal a shard started at 1000
    arr2 = R.ARayShooter.RandomCircle(400 * nm, 110.0, 10, None, R.TGeoTranslation(0, 0, 1600), (0, 0, -1),
                                      first_id=1000)
    np.testing.assert_array_equal(arr2.x, arr.x[1000:1010])


def test_deterministic_shooters():
    arr = R.ARayShooter.Square(400 * nm, 10.0, 3)
    assert len(arr) == 9
    np.testing.assert_allclose(sorted(set(np.round(arr.x, 9))), [-5, 0, 5])
    c = R.ARayShooter.Circle(400 * nm, 10.0, 2, 6)
    assert len(c) == 1 + 6 + 12
    np.testing.assert_allclose(np.hypot(c.x, c.y)[1:7], 5.0)
    rot = R.TGeoRotation("", 0, 90, 0)
    sq = R.ARayShooter.RandomSquare(400 * nm, 2.0, 100, rot, None)
    np.testing.assert_allclose(sq.directions(), np.tile(rot.R @ [0, 0, 1], (100, 1)), atol=1e-15)
    sph = R.ARayShooter.RandomSphere(400 * nm, 50000)
    d = sph.directions()
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-12)
    assert abs(d[:, 2].mean()) < 0.02
    cone = R.ARayShooter.RandomSphericalCone(400 * nm, 20000, 10.0)
    assert np.degrees(np.arccos(cone.dz)).max() <= 10.0 + 1e-9


def test_euler_convention():
    # TGeoRotation(phi, theta, psi) = Rz(phi) Rx(theta) Rz(psi)
    r = R.TGeoRotation("", 90, 0, 0)
    np.testing.assert_allclose(r.R @ [1, 0, 0], [0, 1, 0], atol=1e-15)
    r = R.TGeoRotation("", 0, 90, 0)
    np.testing.assert_allclose(r.R @ [0, 0, 1], [0, -1, 0], atol=1e-15)


def test_boolean_expression_parser():
    a = R.TGeoBBox("pa", 1, 1, 1)
    b = R.TGeoBBox("pb", 2, 2, 2)
    c = R.TGeoBBox("pc", 3, 3, 3)
    t = R.TGeoTranslation("pt", 0, 0, 1).RegisterYourself()
    comp = R.TGeoCompositeShape("pcomp", "pa:pt + pb * pc - pa")
    assert comp.op == N.OP_SUBTRACTION
    assert comp.right is a
    left = comp.left
    assert left.op == N.OP_UNION and left.left is a and left.left_matrix is t
    assert left.right.op == N.OP_INTERSECTION


def test_scene_tuning_set_and_read_back():
    """rbg_scene_set_tuning validates its arguments and rbg_scene_tuning
    reports the tuning (host state only: no device needed)."""
    from robast_gb300 import configs

    man, _ = configs.schwarzschild_couder(n_rays=5)
    h = man.scene.handle
    L = N.lib()
    b, c = C.c_int32(0), C.c_int32(0)
    assert L.rbg_scene_tuning(h, C.byref(b), C.byref(c)) == N.RBG_OK
    assert (b.value, c.value) == (256, 32)  # the lean instance's defaults
    assert L.rbg_scene_set_tuning(h, 128, 8) == N.RBG_OK
    assert L.rbg_scene_tuning(h, C.byref(b), None) == N.RBG_OK and b.value == 128
    assert L.rbg_scene_tuning(h, None, C.byref(c)) == N.RBG_OK and c.value == 8
    for bad in ((64, 8), (512, 8), (128, 33), (128, -1)):
        assert L.rbg_scene_set_tuning(h, *bad) == N.RBG_ERR_ARG
    assert L.rbg_scene_set_tuning(None, 0, 0) == N.RBG_ERR_ARG
    # another scene class runs at its instance's own block size
    man2, _ = configs.davies_cotton(n_rays=5)
    assert L.rbg_scene_tuning(man2.scene.handle, C.byref(b), C.byref(c)) == N.RBG_OK
    assert b.value == 256 and c.value == 32


def test_trace_async_needs_the_scene_on_the_device():
    """rbg_trace_async never uploads (an upload allocates and copies, which
    a graph capture cannot hold): a scene not yet on a device is an argument
    error, and so is reading the status of a scene that never traced."""
    from robast_gb300 import configs

    man, _ = configs.paraboloid(n_rays=5)
    L = N.lib()
    rays, res, opts = N.Rays(), N.Result(), man.trace_options()
    assert L.rbg_trace_async(man.scene.handle, C.byref(rays), C.byref(res), C.byref(opts), None) == N.RBG_ERR_ARG
    assert L.rbg_trace_status(man.scene.handle, None) == N.RBG_ERR_ARG
    assert L.rbg_trace_status(None, None) == N.RBG_ERR_ARG
