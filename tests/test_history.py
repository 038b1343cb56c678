"""Per-ray point/node histories and the ARay node queries
(src/ARay.cxx:42-64, FindNodeStartWith / FindNodeNumberStartWith), used by
the facet-hit map of tutorials/DaviesCotton.C:214-223."""
import numpy as np
import pytest

import oracle_ref
from robast_gb300 import (AMirror, AOpticalComponent, AOpticsManager, ARay, TGeoBBox, TGeoTranslation, configs)


def _nested_manager():
    man = AOpticsManager("m", "nested")
    world = AOpticalComponent("world", TGeoBBox("w", 100, 100, 100))
    man.SetTopVolume(world)
    box = AOpticalComponent("holder", TGeoBBox("h", 10, 10, 10))
    mir = AMirror("mirror", TGeoBBox("mb", 1, 1, 1))
    box.AddNode(mir, 5, TGeoTranslation(0, 0, -2))
    world.AddNode(box, 3, TGeoTranslation(0, 0, 0))
    world.AddNode(box, 7, TGeoTranslation(50, 0, 0))
    man.CloseGeometry()
    return man


def test_node_root_names():
    """TGeoNode names are "<volume>_<copy>", physical ids breadth first."""
    man = _nested_manager()
    assert man.scene.node_root_names() == ["world_1", "holder_3", "holder_7", "mirror_5", "mirror_5"]


def _scalar_find(hist_node, npoints, names, prefix):
    out = np.full(len(npoints), -1, dtype=np.int64)
    for i in range(len(npoints)):
        for k in range(min(int(npoints[i]), hist_node.shape[1]) - 1):
            nd = hist_node[i, k + 1]
            if nd >= 0 and names[nd].startswith(prefix):
                out[i] = k
                break
    return out


def _dc_small(n_rays=3000):
    return configs.davies_cotton(n_rays=n_rays, n_angles=2, n_facets=37)


def test_find_node_number_vectorised_matches_ray_loop():
    man, batch = _dc_small()
    rays = configs.to_array(batch)
    st, ref = oracle_ref.trace(man, rays, threads=4, history=8)
    arr = configs.to_array(batch)
    arr.status, arr.npoints, arr.last_node = ref["status"], ref["npoints"], ref["last_node"]
    arr.hist_xyzt, arr.hist_node = ref["hist_xyzt"], ref["hist_node"]
    arr.node_names = man.scene.node_root_names()
    for prefix in ("mirror", "mirror_1", "focalPlane", "cameraBox", "nothing"):
        got = arr.FindNodeNumberStartWith(prefix)
        np.testing.assert_array_equal(got, _scalar_find(arr.hist_node, arr.npoints, arr.node_names, prefix))
    k = arr.FindNodeNumberStartWith("mirror")
    foc = arr.GetFocused()
    assert len(foc) > 100
    # every focused ray entered the world (the rays start outside it) and
    # then reflected off a facet
    assert (k[foc] == 1).all()
    assert (arr.FindNodeNumberStartWith("world_1", foc) == 0).all()
    nodes = arr.FindNodeStartWith("mirror", foc)
    assert all(arr.node_names[nd].startswith("mirror_") for nd in nodes)
    rows, pts = arr.NodeHitPoints("mirror")
    assert set(foc) <= set(rows)
    # facet hits lie on the dish: inside the 37-facet aperture and below
    # the sagitta of its rim
    r = np.hypot(pts[:, 0], pts[:, 1])
    assert (r < 250).all() and (pts[:, 2] > -1).all() and (pts[:, 2] < 30).all()
    # GetPoint / GetNodeHistory agree with the raw history
    i = int(foc[0])
    np.testing.assert_array_equal(arr.GetPoint(i, 1), arr.hist_xyzt[i, 1])
    assert list(arr.GetNodeHistory(i))[1] == nodes[0]
    assert np.isnan(arr.GetPoint(i, 50)).all()


def test_history_required():
    arr = ARayShooter_square()
    with pytest.raises(RuntimeError):
        arr.FindNodeNumberStartWith("mirror")


def ARayShooter_square():
    from robast_gb300 import ARayShooter
    return ARayShooter.Square(400e-7, 10.0, 3)


@pytest.mark.gpu
def test_history_api_gpu_matches_oracle():
    man, batch = _dc_small()
    st, ref = oracle_ref.trace(man, configs.to_array(batch), threads=4, history=8)
    arr = configs.to_array(batch)
    man.TraceNonSequential(arr, history=8)
    k_ref = _scalar_find(ref["hist_node"], ref["npoints"], man.scene.node_root_names(), "mirror")
    k = arr.FindNodeNumberStartWith("mirror")
    assert (k == k_ref).mean() >= 0.999
    same = (k == k_ref) & (k >= 0)
    rows, pts = arr.NodeHitPoints("mirror", np.nonzero(same)[0])
    np.testing.assert_allclose(pts[:, :3], ref["hist_xyzt"][rows, k_ref[rows] + 1, :3], rtol=0, atol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_history_tail_is_defined(precision):
    """Slots past a ray's npoints read node -3 and point 0 whatever the
    device memory held before (recycled allocations), in both tracers, and
    the whole history equals the oracle's."""
    import torch

    from robast_gb300 import _native as N
    from robast_gb300 import device

    man, batch = configs.schwarzschild_couder(n_rays=20000, angles=(0.0, 4.0), seed=9)
    n, cap = len(batch["x"]), 6
    res = device.alloc_result(n, "cuda:0", cap)
    res["hist_node"].fill_(2)  # stale ids that name a real node
    res["hist_xyzt"].fill_(float("nan"))
    res, st = device.trace(man, device.to_device(batch), res,
                           precision=N.PREC_FP64 if precision == "fp64" else N.PREC_MIXED)
    torch.cuda.synchronize()
    assert st == 0
    npts = res["npoints"].cpu().numpy()
    hn = res["hist_node"].cpu().numpy()
    hx = res["hist_xyzt"].cpu().numpy()
    tail = np.arange(cap)[None, :] >= npts[:, None]
    assert tail.any()
    assert (hn[tail] == -3).all()
    assert (hx[tail] == 0).all()
    ost, ref = oracle_ref.trace(man, configs.to_array(batch), threads=8, history=cap)
    assert ost == 0
    np.testing.assert_array_equal(hn, ref["hist_node"].reshape(n, cap))
    np.testing.assert_allclose(hx, ref["hist_xyzt"].reshape(n, cap, 4), rtol=1e-9, atol=1e-9)


@pytest.mark.gpu
def test_single_ray_keeps_full_history():
    man, _ = configs.paraboloid(n_rays=4, angles=(0.0,))
    # outside the 30 cm obscuration disk in front of the focal plane
    ray = ARay(0, 400e-7, 50.0, 0.0, 1600.0, 0.0, 0.0, 0.0, -1.0)
    man.TraceNonSequential(ray)
    assert ray.IsFocused()
    assert len(ray.points) == ray.GetNpoints() == len(ray.nodes) + 1
    assert ray.FindNodeStartWith("mirror") == "mirror_1"
    k = ray.FindNodeNumberStartWith("mirror")
    assert k >= 0 and ray.FindNodeNumberStartWith("focal") > k
    # the mirror hit is on the paraboloid z = r^2 / 4f below the focus
    x, y, z, _ = ray.GetPoint(k + 1)
    assert abs(z - (x * x + y * y) / (4 * 800.0)) < 1e-3


def test_ray_setters_and_node_lookup():
    ray = ARay(0, 400e-7, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, -1.0)
    for set_, check in ((ray.Absorb, ray.IsAbsorbed), (ray.Exit, ray.IsExited), (ray.Focus, ray.IsFocused),
                        (ray.Stop, ray.IsStopped), (ray.Suspend, ray.IsSuspended)):
        set_()
        assert check()
    ray.SetLambda(500e-7)
    assert ray.GetLambda() == 500e-7
    ray.node_names = ["world_1", "mirror_3"]
    ray.nodes = [0, 1, -1]
    assert ray.FindNode("mirror_3") == "mirror_3" and ray.FindNode("mirror") is None
    assert ray.FindNodeStartWith("mir") == "mirror_3" and ray.FindNodeNumberStartWith("mir") == 1
    assert ray.GetNodeHistory() == [0, 1, -1]


def test_manager_classification_and_border_components():
    from robast_gb300 import ABorderSurfaceCondition, AFocalSurface, ALens, AObscuration
    man = _nested_manager()
    world = man.GetTopVolume()
    mir = AMirror("m2", TGeoBBox("b2", 1, 1, 1))
    obs = AObscuration("o", TGeoBBox("b3", 1, 1, 1))
    plain = AOpticalComponent("c", TGeoBBox("b4", 1, 1, 1))
    assert man.IsObscuration(obs) and not man.IsObscuration(mir)
    assert man.IsOpticalComponent(plain) and not man.IsOpticalComponent(mir)
    cond = ABorderSurfaceCondition(world, mir)
    assert cond.GetComponent1() is world and cond.GetComponent2() is mir
