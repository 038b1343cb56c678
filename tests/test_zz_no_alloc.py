"""rbg_trace_noalloc: the trace entry point that allocates no device memory.

It is for callers that cannot let a library allocate or free GPU memory
(a real-time camera trigger chain or a serving process that owns all device
memory in a fixed budget, where cudaMalloc may fail and cudaFree would
synchronise the device).  Its scratch -- scene tables, error word, ray-queue
counter -- lives in a fixed 4 MiB static device array.  Its results must
equal those of rbg_trace (same persistent kernel, same Philox draws) on two
calls in a row, since every call reuses the array left by the previous one.

This file is named to be collected last: it runs after every other test
and also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import robast_gb300 as R
from robast_gb300 import _native as N
from robast_gb300 import configs

pytestmark = pytest.mark.gpu

RTOL = 1e-6  # the tolerance the parity tests use for positions


def _noalloc():
    L = N.lib()
    f = L.rbg_trace_noalloc
    f.argtypes = [C.c_void_p, C.POINTER(N.Rays), C.POINTER(N.Result), C.POINTER(N.TraceOpts), C.c_void_p]
    f.restype = C.c_int
    return f


def _noalloc_trace(man, rays, res):
    import torch

    from robast_gb300 import device

    scene = man._ensure_scene()
    rs = device._rays_struct(rays)
    rr = device._result_struct(res)
    opts = man.trace_options(N.PREC_MIXED)
    st = torch.cuda.current_stream().cuda_stream
    return _noalloc()(scene.handle, C.byref(rs), C.byref(rr), C.byref(opts), C.c_void_p(st))


def _host(res):
    return {k: v.cpu().numpy() for k, v in res.items()}


NM = 1e-7


@pytest.mark.parametrize("name,kw", [
    ("schwarzschild_couder", dict(n_rays=20000)),
    ("paraboloid", dict(n_rays=20000)),
    ("light_guide", dict(n_rays=8000, n_variants=2)),
    # precalculated thin-film tables: the first call fills them inside the
    # static array and keeps a host copy for the calls after it
    ("schmidt_cassegrain", dict(n_rays=6000, n_samples=2,
                                coating_table=(32, 340 * NM, 660 * NM, 24, 0.0, 0.6))),
])
def test_noalloc_matches_trace_twice(name, kw):
    """The no-allocation call runs first, on a scene no other entry point
    has touched (its tables and its thin-film table fill are set up by
    rbg_trace_noalloc itself, twice in a row); the reference is rbg_trace
    on a second, identical scene afterwards."""
    import torch

    from robast_gb300 import device

    man, batch = configs.CONFIGS[name](**kw)
    rays = device.to_device(batch)
    n = len(batch["x"])
    got_calls = []
    for call in range(2):
        res = device.alloc_result(n)
        for v in res.values():
            v.fill_(7)  # stale contents must be overwritten
        st = _noalloc_trace(man, rays, res)
        torch.cuda.synchronize()
        assert st == N.RBG_OK, (call, N.status_string(st))
        got_calls.append(_host(res))
    man2, batch2 = configs.CONFIGS[name](**kw)
    ref, st = device.trace(man2, device.to_device(batch2), precision=N.PREC_MIXED)
    assert st == 0
    ref = _host(ref)
    for call, got in enumerate(got_calls):
        for k in ("status", "npoints", "last_node"):
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f"call {call}: {k}")
        for k in ("x", "y", "z", "t", "dx", "dy", "dz"):
            np.testing.assert_allclose(got[k], ref[k], rtol=RTOL, atol=1e-9, err_msg=f"call {call}: {k}")


def test_noalloc_rejects_scene_beyond_limit():
    from robast_gb300 import device

    man = R.AOpticsManager()
    world = R.AOpticalComponent("world", R.TGeoBBox("wb", 5e4, 5e4, 10))
    man.SetTopVolume(world)
    box = R.AObscuration("tile", R.TGeoBBox("tb", 1, 1, 1))
    for i in range(30000):  # 30000 nodes x 176 B > 4 MiB
        world.AddNode(box, i + 1, R.TGeoTranslation(3.0 * (i % 1000) - 1500, 3.0 * (i // 1000), 0))
    man.CloseGeometry()
    rays = device.to_device({"x": np.zeros(4), "y": np.zeros(4), "z": np.full(4, 5.0), "dx": np.zeros(4),
                             "dy": np.zeros(4), "dz": np.full(4, -1.0), "lam": np.full(4, 4e-5)})
    res = device.alloc_result(4)
    st = _noalloc_trace(man, rays, res)
    assert st == N.RBG_ERR_TOO_LARGE
    assert "no-allocation" in N.status_string(st)


def test_noalloc_rejects_fp64_request():
    from robast_gb300 import device

    man, batch = configs.paraboloid(n_rays=16)
    rays = device.to_device(batch)
    res = device.alloc_result(16)
    scene = man._ensure_scene()
    opts = man.trace_options(N.PREC_FP64)
    st = _noalloc()(scene.handle, C.byref(device._rays_struct(rays)), C.byref(device._result_struct(res)),
                    C.byref(opts), None)
    assert st == N.RBG_ERR_UNSUPPORTED
