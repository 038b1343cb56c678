"""The allocation contract of the trace entry point: after rbg_scene_reserve
has made the scene's device allocations, rbg_trace allocates nothing, for
batches up to the reserved size (spatial take-up order) and beyond it
(input order, the same results).  The adjoint keeps its parameters in the
launch and its skip counter in the scene's own block, so it allocates
nothing either.  Free device memory is read with cudaMemGetInfo (through
torch) around the calls, after a warm-up that has loaded every kernel."""
import numpy as np
import pytest

from robast_gb300 import configs

pytestmark = pytest.mark.gpu


def _free():
    import torch

    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_trace_allocates_nothing_after_reserve():
    import torch

    from robast_gb300 import _native as N
    from robast_gb300 import device

    n = 1 << 19
    man, batch = configs.schwarzschild_couder(n_rays=2 * n, seed=21)
    big = device.to_device(batch)
    half = {k: v[:n] for k, v in big.items()}
    warm = {k: v[: 1 << 15] for k, v in big.items()}
    res_big = device.alloc_result(2 * n)
    res_half = device.alloc_result(n)
    res_warm = device.alloc_result(1 << 15)
    device.reserve(man, n)
    for p in (N.PREC_MIXED, N.PREC_FP64):
        device.trace(man, warm, res_warm, precision=p, workspace_buf=None)  # loads every kernel once
    before = _free()
    out = {}
    for p in (N.PREC_MIXED, N.PREC_FP64):
        _, st = device.trace(man, half, res_half, precision=p, workspace_buf=None)  # reserved size: spatial order
        assert st == 0
        out[p] = {k: v.cpu().numpy() for k, v in res_half.items()}
        _, st = device.trace(man, big, res_big, precision=p, workspace_buf=None)  # beyond it: input order
        assert st == 0
    assert _free() == before
    # beyond the reservation the results are those of the first n rays traced alone
    for p in (N.PREC_MIXED, N.PREC_FP64):
        device.trace(man, big, res_big, precision=p, workspace_buf=None)
        for k in ("status", "npoints", "last_node", "x", "y", "z", "dx", "dy", "dz"):
            np.testing.assert_array_equal(res_big[k][:n].cpu().numpy(), out[p][k], err_msg=k)
    torch.cuda.synchronize()


def test_adjoint_allocates_nothing():
    import torch

    from robast_gb300 import _native as N
    from robast_gb300 import adjoint as A
    from robast_gb300 import device

    build = A.sc_builder()
    man, specs = build(A.sc_parameters())
    _, batch = configs.schwarzschild_couder(n_rays=40_000, seed=22)
    rays = device.to_device(batch)
    res, st = A.trace_with_history(man, rays)
    assert st == 0
    f = (res["status"] == N.RBG_FOCUS).double()
    gx, gy = 2 * res["x"] * f, 2 * res["y"] * f
    g1, _ = A.vjp(man, res, specs, gx, gy)  # warm-up: loads the kernel
    before = _free()
    g2, _ = A.vjp(man, res, specs, gx, gy)
    assert _free() == before
    # the same gradient (its per-warp partial sums meet in atomic order)
    torch.testing.assert_close(g1, g2, rtol=1e-12, atol=0)
