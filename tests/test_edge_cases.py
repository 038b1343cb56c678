"""Edge cases of rbg_trace on the GPU: invalid rays, launch shape, batch
splits, side streams, optional outputs, and rays that start outside the
top volume.  Per-ray results depend only on (seed, global ray id), so all
of these must agree bit for bit with a plain trace of the same rays."""
import ctypes as C

import numpy as np
import pytest

import oracle_ref
from robast_gb300 import _native as N
from robast_gb300 import configs

pytestmark = pytest.mark.gpu

FIELDS = ("status", "npoints", "last_node", "x", "y", "z", "t", "dx", "dy", "dz")


def _trace(man, batch, precision, offset=0, block_size=0, stream=None, fields=FIELDS):
    import torch

    from robast_gb300 import device

    rays = device.to_device(batch, "cuda:0")
    res = device.alloc_result(len(batch["x"]), "cuda:0")
    rr = device._result_struct(res)
    for f in FIELDS:
        if f not in fields:
            setattr(rr, f, None)
    opts = man.trace_options(precision)
    opts.ray_id_offset = offset
    opts.block_size = block_size
    st = stream if stream is not None else torch.cuda.current_stream()
    with torch.cuda.stream(st):
        status = N.lib().rbg_trace(man._ensure_scene().handle, C.byref(device._rays_struct(rays)), C.byref(rr),
                                   C.byref(opts), C.c_void_p(st.cuda_stream))
    st.synchronize()
    return status, {k: res[k].cpu().numpy() for k in fields}


def _same(a, b, idx=None):
    for k in a:
        if k in b:
            x, y = (a[k], b[k]) if idx is None else (a[k][idx], b[k][idx])
            np.testing.assert_array_equal(x, y, err_msg=k)


PRECS = [N.PREC_FP64, N.PREC_MIXED]


@pytest.mark.parametrize("prec", PRECS)
def test_invalid_rays_are_reported_and_isolated(prec):
    man, batch = configs.davies_cotton(n_rays=4000, n_angles=2)
    bad = {5: ("x", np.nan), 17: ("dx", 0.0), 33: ("dz", np.inf), 34: ("y", -np.inf)}
    dirty = {k: v.copy() for k, v in batch.items()}
    for i, (f, v) in bad.items():
        if f == "dx":
            dirty["dx"][i] = dirty["dy"][i] = dirty["dz"][i] = 0.0
        else:
            dirty[f][i] = v
    st, got = _trace(man, dirty, prec)
    assert st == N.RBG_ERR_NAN
    idx = np.array(sorted(bad))
    assert (got["status"][idx] == N.RBG_RUN).all() and (got["npoints"][idx] == 1).all()
    st0, ref = _trace(man, batch, prec)
    assert st0 == N.RBG_OK
    good = np.setdiff1d(np.arange(len(batch["x"])), idx)
    _same(got, ref, good)


@pytest.mark.parametrize("block", [32, 64, 96])
def test_fp64_launch_shape_does_not_change_results(block):
    man, batch = configs.davies_cotton(n_rays=5000, n_angles=2)
    _, ref = _trace(man, batch, N.PREC_FP64)
    _, got = _trace(man, batch, N.PREC_FP64, block_size=block)
    _same(got, ref)


@pytest.mark.parametrize("prec", PRECS)
def test_split_batches_with_offsets_match_whole(prec):
    man, batch = configs.davies_cotton(n_rays=6000, n_angles=2)
    _, whole = _trace(man, batch, prec)
    cut = 2345
    _, a = _trace(man, {k: v[:cut] for k, v in batch.items()}, prec, offset=0)
    _, b = _trace(man, {k: v[cut:] for k, v in batch.items()}, prec, offset=cut)
    _same({k: np.concatenate([a[k], b[k]]) for k in a}, whole)
    # a wrong offset changes the random draws (roughness): the results differ
    _, c = _trace(man, {k: v[cut:] for k, v in batch.items()}, prec, offset=0)
    assert not np.array_equal(c["x"], b["x"])


@pytest.mark.parametrize("prec", PRECS)
def test_side_stream_and_optional_outputs(prec):
    import torch

    man, batch = configs.schwarzschild_couder(n_rays=5000, perturb=0.0)
    _, ref = _trace(man, batch, prec)
    _, side = _trace(man, batch, prec, stream=torch.cuda.Stream())
    _same(side, ref)
    st, some = _trace(man, batch, prec, fields=("status", "x"))
    assert st == N.RBG_OK
    _same(some, ref)


@pytest.mark.parametrize("prec", PRECS)
def test_rays_starting_outside_the_top_volume(prec):
    man, batch = configs.paraboloid(n_rays=4000, seed=5)
    n = len(batch["x"])
    b = {k: v.copy() for k, v in batch.items()}
    # half of the rays start 10 m above the 20 m world box, half of those point away
    b["z"][: n // 2] = 3000.0
    b["dz"][: n // 4] = -b["dz"][: n // 4]
    st, got = _trace(man, b, prec)
    assert st == N.RBG_OK
    ost, ref = oracle_ref.trace(man, configs.to_array(b), threads=8)
    assert ost == 0
    for k in ("status", "npoints", "last_node"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    for k in ("x", "y", "z"):
        np.testing.assert_allclose(got[k], ref[k], rtol=1e-6, atol=1e-6)
    assert (got["status"][: n // 4] == N.RBG_EXIT).all()
    assert (got["status"][n // 4: n // 2] == N.RBG_FOCUS).mean() > 0.3


@pytest.mark.parametrize("prec", PRECS)
def test_host_pipeline_matches_device_trace(prec):
    """rbg_trace_host runs the batch as chunks of 2^21 rays over two streams
    with per-chunk ray-id offsets: two chunks (the second partial), with
    histories, must equal one device-buffer trace bit for bit, and a second
    call reusing the workspace must equal the first."""
    import torch

    from robast_gb300 import device
    from robast_gb300.manager import make_result

    n = (1 << 21) + 3001
    man, batch = configs.davies_cotton(n_rays=n, n_angles=2)
    hist = 2
    rays = device.to_device(batch, "cuda:0")
    ref_res = device.alloc_result(n, "cuda:0", hist)
    ref_res, st = device.trace(man, rays, ref_res, precision=prec)
    torch.cuda.synchronize()
    assert st == N.RBG_OK
    ref = {k: v.cpu().numpy() for k, v in ref_res.items()}
    arr = configs.to_array(batch)
    dp = C.POINTER(C.c_double)
    rs = N.Rays(n, *(getattr(arr, f).ctypes.data_as(dp) for f in ("x", "y", "z", "t", "dx", "dy", "dz", "lam")))
    opts = man.trace_options(prec)
    for call in range(2):
        rr, got = make_result(n, hist)
        st = N.lib().rbg_trace_host(man._ensure_scene().handle, C.byref(rs), C.byref(rr), C.byref(opts))
        assert st == N.RBG_OK, (call, N.status_string(st))
        # one trace per chunk; the first chunk also runs the seven kernels
        # of its spatial take-up order (the 3001-ray second chunk is below
        # the 2^14 rays that get one)
        want = 2 + 7
        assert N.lib().rbg_last_launch_count(man.scene.handle) == want
        for k in FIELDS:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f"call {call}: {k}")
        valid = np.arange(hist)[None, :] < np.minimum(ref["npoints"], hist)[:, None]
        np.testing.assert_array_equal(got["hist_node"][valid], ref["hist_node"][valid])
        np.testing.assert_array_equal(got["hist_xyzt"][valid], ref["hist_xyzt"][valid])


@pytest.mark.parametrize("name", ["schwarzschild_couder", "davies_cotton", "light_guide"])
def test_compaction_threshold_does_not_change_results(name):
    """The mixed tracer's refill threshold only changes which lanes carry
    which rays; every ray's result depends on (seed, ray id) alone."""
    kw = {"light_guide": dict(n_rays=6000, n_variants=2)}.get(name, dict(n_rays=6000))
    man, batch = configs.CONFIGS[name](**kw)
    results = []
    for c in (1, 7, 32):
        man.compaction = c
        st, got = _trace(man, batch, N.PREC_MIXED)
        assert st == N.RBG_OK
        results.append(got)
    for got in results[1:]:
        _same(got, results[0])


def test_autotune_picks_a_candidate_and_keeps_results():
    import torch

    from robast_gb300 import device

    man, batch = configs.schwarzschild_couder(n_rays=20000, seed=9)
    st, ref = _trace(man, batch, N.PREC_MIXED)
    assert st == N.RBG_OK
    rays = device.to_device(batch, "cuda:0")
    res = device.alloc_result(len(batch["x"]), "cuda:0")
    assert device.tuning(man) == (256, 32)  # the lean instance's defaults before tuning
    chosen = device.autotune(man, rays, res)
    torch.cuda.synchronize()
    assert chosen in (1, 8, 16, 32)
    # the tuned pair: a block size the lean instance is compiled for
    block, thr = device.tuning(man)
    assert block in (128, 256) and thr == chosen
    # a tuning set directly is the one reported, and changes no result
    device.set_tuning(man, 128, 1)
    assert device.tuning(man) == (128, 1)
    assert man.scene is not None
    tuned = {k: res[k].cpu().numpy() for k in FIELDS}
    _same(tuned, ref)
    st, after = _trace(man, batch, N.PREC_MIXED)
    assert st == N.RBG_OK
    _same(after, ref)


def test_trace_async_in_a_cuda_graph():
    """rbg_trace_async puts the whole trace (take-up order and persistent
    tracer) on the stream without reading anything back, so a CUDA graph
    captures it; replays give rbg_trace's results, and rbg_trace_status
    reads the status afterwards."""
    import torch

    from robast_gb300 import device

    man, batch = configs.schwarzschild_couder(n_rays=60000, seed=9)
    n = len(batch["x"])
    rays = device.to_device(batch, "cuda:0")
    device.reserve(man, n)
    ref, st = device.trace(man, rays, precision=N.PREC_MIXED)
    assert st == N.RBG_OK
    ref = {k: ref[k].cpu().numpy() for k in FIELDS}
    res = device.alloc_result(n, "cuda:0")
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):  # warm-up on the capture stream
        device.trace_async(man, rays, res, precision=N.PREC_MIXED, stream=side)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        device.trace_async(man, rays, res, precision=N.PREC_MIXED, stream=side)
    for _ in range(2):
        for v in res.values():
            v.fill_(7)
        graph.replay()
        torch.cuda.synchronize()
        assert device.status(man) == N.RBG_OK
        _same({k: res[k].cpu().numpy() for k in FIELDS}, ref)
