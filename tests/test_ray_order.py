"""The mixed tracer's take-up order (rbg_trace_opts.ray_order): grouping the
rays of a batch by the Morton cell of their start point changes which rays
share a warp, never a result -- every ray keeps its index for its inputs,
outputs and Philox draws, so deterministic and stochastic scenes alike give
bit-identical outputs in spatial and in input order, through the device
call and through the host pipeline."""
import numpy as np
import pytest

from robast_gb300 import _native as N
from robast_gb300 import configs

pytestmark = pytest.mark.gpu

FIELDS = ("status", "npoints", "last_node", "x", "y", "z", "t", "dx", "dy", "dz")


def _device(man, batch, order, history=0):
    import torch

    from robast_gb300 import device

    man.ray_order = order
    rays = device.to_device(batch, "cuda:0")
    res = device.alloc_result(len(batch["x"]), "cuda:0", history)
    res, st = device.trace(man, rays, res, precision=N.PREC_MIXED)
    torch.cuda.synchronize()
    return st, {k: v.cpu().numpy() for k, v in res.items()}


@pytest.mark.parametrize("name,n", [("schwarzschild_couder", 200_000), ("davies_cotton", 100_000),
                                    ("light_guide", 100_000), ("schmidt_cassegrain", 100_000),
                                    ("paraboloid", 100_000)])
def test_spatial_order_changes_no_result(name, n):
    man, batch = configs.CONFIGS[name](n_rays=n)
    st0, a = _device(man, batch, N.ORDER_INPUT)
    st1, b = _device(man, batch, N.ORDER_SPATIAL)
    assert st0 == st1
    for f in FIELDS:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)


def test_spatial_order_histories_and_host_pipeline():
    man, batch = configs.davies_cotton(n_rays=60_000, n_angles=3)
    _, a = _device(man, batch, N.ORDER_INPUT, history=6)
    _, b = _device(man, batch, N.ORDER_SPATIAL, history=6)
    np.testing.assert_array_equal(a["hist_node"], b["hist_node"])
    np.testing.assert_array_equal(a["hist_xyzt"], b["hist_xyzt"])
    arr = configs.to_array(batch)
    man.ray_order = N.ORDER_SPATIAL
    man.TraceNonSequential(arr, precision=N.PREC_MIXED)
    for f in ("status", "npoints", "last_node"):
        np.testing.assert_array_equal(getattr(arr, f), a[f])
    np.testing.assert_array_equal(arr.x, a["x"])

