"""The product's scene flattening (rbg_scene_create, C++) against the
independent restatement the oracle traces (tests/flat_ref.py), field by
field, for the five telescope configurations and the shape scenes of the
other tests: the physical tree, every node's local -> master matrix, the
canonical parameters of every shape (AGeoAsphericDisk's ComputeBBox
origin and half height, Winston cone dimensions, paraboloid coefficients,
phi ranges) and the bounding boxes (the product's must enclose the shape).
A flattening error injected on the host -- a placement matrix with two
Euler angles swapped, a Winston cone with the wrong number of sides -- must
fail the comparison.  CPU only.
"""
import math

import numpy as np
import pytest

import flat_ref
import robast_gb300 as R
from robast_gb300 import _native as N
from robast_gb300 import configs


def compare_flat(prod, ind, canon):
    """List of differences between the product's flat scene and the
    independent one (empty when they agree)."""
    bad = []
    if prod.n_nodes != ind.n_nodes:
        return [f"node count {prod.n_nodes} vs {ind.n_nodes}"]
    for i in range(prod.n_nodes):
        a, b = prod.nodes[i], ind.nodes[i]
        for f in ("parent", "volume", "shape", "kind", "child_begin", "child_count"):
            if getattr(a, f) != getattr(b, f):
                bad.append(f"node {i} {f} {getattr(a, f)} vs {getattr(b, f)}")
        ma, mb = np.array(a.m[:]), np.array(b.m[:])
        if not np.allclose(ma, mb, rtol=1e-12, atol=1e-9):
            bad.append(f"node {i} matrix {ma} vs {mb}")
        for k in range(3):
            # the product's box may be padded, but must hold the shape
            if not (a.lo[k] <= b.lo[k] + 1e-7 * max(1.0, abs(b.lo[k])) and
                    a.hi[k] >= b.hi[k] - 1e-7 * max(1.0, abs(b.hi[k]))):
                bad.append(f"node {i} box axis {k}: [{a.lo[k]}, {a.hi[k]}] misses [{b.lo[k]}, {b.hi[k]}]")
    if [prod.children[i] for i in range(prod.n_children)] != [ind.children[i] for i in range(ind.n_children)]:
        bad.append("children lists differ")
    for sid in range(prod.n_shapes):
        sa = prod.shapes[sid]
        if sa.type == N.SHAPE_COMPOSITE:
            got = np.array([prod.params[sa.param_offset + k] for k in range(24)])
        else:
            got = np.array([prod.params[sa.param_offset + k] for k in range(len(canon[sid]))])
        want = np.array(canon[sid], dtype=float)
        if got.shape != want.shape or not np.allclose(got, want, rtol=1e-12, atol=1e-12, equal_nan=True):
            bad.append(f"shape {sid} (type {sa.type}) params {got} vs {want}")
    return bad


def _check(man):
    scene = man._ensure_scene()
    ind = flat_ref.IndependentFlat(scene)
    diffs = compare_flat(scene.flat, ind.flat, ind.canonical)
    assert not diffs, "\n".join(diffs[:10])
    return scene, ind


SMALL = {
    "paraboloid": dict(n_rays=8),
    "davies_cotton": dict(n_rays=8),
    "schwarzschild_couder": dict(n_rays=8),
    "light_guide": dict(n_rays=8, n_variants=4),
    "schmidt_cassegrain": dict(n_rays=8, n_samples=4),
}


@pytest.mark.parametrize("name", sorted(SMALL))
def test_configurations_flatten_alike(name):
    man, _ = configs.CONFIGS[name](**SMALL[name])
    _check(man)


def test_misaligned_secondary_flattens_alike():
    man, _ = configs.schwarzschild_couder(n_rays=8, secondary_shift=(0.3, -0.2, 0.5),
                                          secondary_tilt=(4e-4, 3e-4, 1e-4))
    _check(man)


def _shape_zoo():
    man = R.AOpticsManager()
    world = R.AOpticalComponent("world", R.TGeoBBox("wb", 500, 500, 500))
    man.SetTopVolume(world)
    shapes = [
        R.TGeoTubeSeg("ts", 1, 3, 2, 300, 60),
        R.TGeoSphere("sp", 2, 5, 20, 140, -30, 200),
        R.TGeoParaboloid("pa", 0.5, 4, 2),
        R.AGeoWinstonConePoly("wp", 2.5, 1.25, 6),
        R.AGeoWinstonConePoly("wq", 1.0, 2.2, 4),
        R.AGeoWinstonCone2D("w2", 3.0, 1.0, 5.0),
    ]
    asph = R.AGeoAsphericDisk("as", 5, 1e-3, -2, -2e-3, 8, 12)  # z1 > z2, rmin > rmax: reordered
    asph.SetPolynomials(2, [1e-4, -3e-7], 1, [2e-5])
    asph.SetConicConstants(-0.5, 0.2)
    shapes.append(asph)
    pg = R.TGeoPgon("pg", 15, 330, 5, 3)
    pg.DefineSection(0, -2, 0.5, 2)
    pg.DefineSection(1, 0, 0, 3)
    pg.DefineSection(2, 2, 1, 2.5)
    shapes.append(pg)
    for i, s in enumerate(shapes):
        rot = R.TGeoRotation(f"r{i}", 10 * i, 25 + 7 * i, -15 * i)
        world.AddNode(R.AOpticalComponent(f"v{i}", s), 1, R.TGeoCombiTrans(20.0 * i, -5.0 * i, 3.0, rot))
    man.CloseGeometry()
    return man


def test_shape_zoo_flattens_alike():
    _check(_shape_zoo())


def test_euler_angles_follow_root():
    """TGeoRotation(phi, theta, psi) = Rz(phi) Rx(theta) Rz(psi) (ROOT's
    x-convention), and RotateX/Y/Z multiply from the left (a rotation
    about the mother's axis)."""
    def rz(a):
        c, s = math.cos(math.radians(a)), math.sin(math.radians(a))
        return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])

    def rx(a):
        c, s = math.cos(math.radians(a)), math.sin(math.radians(a))
        return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])

    def ry(a):
        c, s = math.cos(math.radians(a)), math.sin(math.radians(a))
        return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])

    r = R.TGeoRotation("e", 30, 50, -70)
    np.testing.assert_allclose(r.R, rz(30) @ rx(50) @ rz(-70), atol=1e-15)
    r.RotateX(12)
    r.RotateY(-8)
    r.RotateZ(5)
    np.testing.assert_allclose(r.R, rz(5) @ ry(-8) @ rx(12) @ rz(30) @ rx(50) @ rz(-70), atol=1e-15)


def _product_flat(desc):
    import ctypes as C

    h = C.c_void_p()
    N.check(N.lib().rbg_scene_create(C.byref(desc), C.byref(h)), "rbg_scene_create")
    f = N.FlatScene()
    N.check(N.lib().rbg_scene_flat(h, C.byref(f)), "rbg_scene_flat")
    return h, f


def test_injected_flattening_errors_are_caught():
    """Errors made on the host in the description the product flattens,
    while the independent flattening reads the intended one: a placement
    whose Euler angles theta and psi were swapped, and a Winston cone with
    the wrong number of polygon sides."""
    man, _ = configs.schwarzschild_couder(n_rays=8)
    scene = man._ensure_scene()
    good = flat_ref.IndependentFlat(scene)
    desc = scene.desc
    mi = desc.n_matrices  # the two rotations go after the existing matrices
    k = next(i for i in range(desc.n_placements) if desc.volumes[desc.placements[i].daughter].kind == N.KIND_MIRROR)
    want = R.TGeoRotation("", 10.0, 0.3, 0.2).R
    swapped = R.TGeoRotation("", 10.0, 0.2, 0.3).R
    assert not np.allclose(want, swapped)
    import ctypes as C

    mats = [desc.matrices[j] for j in range(12 * desc.n_matrices)]
    for R_ in (want, swapped):
        mats += list(R_.reshape(-1)) + [0.0, 0.0, 0.0]
    arr = (C.c_double * len(mats))(*mats)
    desc.matrices, desc.n_matrices = C.cast(arr, C.POINTER(C.c_double)), len(mats) // 12
    old = desc.placements[k].matrix
    desc.placements[k].matrix = mi  # the intended rotation
    good = flat_ref.IndependentFlat(scene)
    desc.placements[k].matrix = mi + 1  # the product gets the swapped one
    h, bad = _product_flat(desc)
    assert compare_flat(bad, good.flat, good.canonical), "a swapped Euler angle went unnoticed"
    N.lib().rbg_scene_destroy(h)
    desc.placements[k].matrix = mi
    h, ok = _product_flat(desc)
    assert not compare_flat(ok, good.flat, good.canonical)
    N.lib().rbg_scene_destroy(h)
    desc.placements[k].matrix = old

    man2 = R.AOpticsManager()
    w = R.AOpticalComponent("w", R.TGeoBBox("wb", 50, 50, 50))
    man2.SetTopVolume(w)
    w.AddNode(R.AOpticalComponent("c", R.AGeoWinstonConePoly("wc", 2.5, 1.25, 6)), 1)
    man2.CloseGeometry()
    s2 = man2._ensure_scene()
    ind2 = flat_ref.IndependentFlat(s2)
    sh = next(i for i in range(s2.desc.n_shapes) if s2.desc.shapes[i].type == N.SHAPE_WINSTON_POLY)
    s2.desc.params[s2.desc.shapes[sh].param_offset + 2] = 4.0
    h, f2 = _product_flat(s2.desc)
    assert compare_flat(f2, ind2.flat, ind2.canonical), "a wrong polygon order went unnoticed"
    N.lib().rbg_scene_destroy(h)


@pytest.mark.parametrize("name", sorted(SMALL))
def test_oracle_agrees_on_both_flattenings(name):
    """The oracle traces the same rays through the product's flattening and
    through the independent one: every fate, point count and last node
    agrees, and the end points to rounding (the two compose their matrices
    and derived constants in different order)."""
    import oracle_ref

    kw = dict(SMALL[name])
    kw["n_rays"] = 3000
    man, batch = configs.CONFIGS[name](**kw)
    arr = configs.to_array(batch)
    st1, a = oracle_ref.trace(man, arr, threads=4, flat="product")
    st2, b = oracle_ref.trace(man, configs.to_array(batch), threads=4, flat="independent")
    assert st1 == st2 == 0
    for k in ("status", "npoints", "last_node"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    for k in ("x", "y", "z", "dx", "dy", "dz"):
        np.testing.assert_allclose(a[k], b[k], rtol=1e-9, atol=1e-9, err_msg=k)
