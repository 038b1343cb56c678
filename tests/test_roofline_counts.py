"""The counting build of the mixed tracer (rbg_trace_count_events), whose
event tallies are the numerator of the bench's FP64- and FP32-pipe roofline
fractions: it traces the same rays to the same results as rbg_trace, and
its counts agree with what the results say about the work done."""
import numpy as np
import pytest

from robast_gb300 import configs

pytestmark = pytest.mark.gpu


def test_counting_build_traces_the_same_rays():
    import torch

    from robast_gb300 import _native as N
    from robast_gb300 import device

    man, batch = configs.schwarzschild_couder(n_rays=60_000, seed=17)
    rays = device.to_device(batch)
    n = len(batch["x"])
    ref, st = device.trace(man, rays, precision=N.PREC_MIXED)
    assert st == 0
    ref = {k: v.cpu().numpy() for k, v in ref.items()}
    res = device.alloc_result(n)
    counts, f64, f32 = device.count_events(man, rays, res)
    torch.cuda.synchronize()
    got = {k: v.cpu().numpy() for k, v in res.items()}
    for k in ("status", "npoints", "last_node", "x", "y", "z", "dx", "dy", "dz"):
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    c = dict(zip(device.EVENT_KINDS, counts))
    assert c["ray"] == n
    # every boundary step adds one point; a step from inside a mirror adds none
    pts = int((ref["npoints"] - 1).sum())
    assert pts <= c["segment"] <= pts + n
    # a focused ray of the two-mirror telescope reflects twice
    assert c["reflect"] >= 2 * int((ref["status"] == N.RBG_FOCUS).sum())
    assert c["polish"] > 0 and c["newton32"] > 0 and c["horner64"] > 0
    assert f64 > 0 and f32 > 0


def test_counting_build_refuses_other_scenes():
    from robast_gb300 import _native as N
    from robast_gb300 import device

    man, batch = configs.paraboloid(n_rays=1000)
    with pytest.raises(N.NativeError):
        device.count_events(man, device.to_device(batch))
