"""Rays grazing the rims of the Schwarzschild-Couder mirrors, the focal
surface and its obscuration, traced by both GPU tracers and checked ray by
ray against the FP64 oracle: fate, point count and last node exactly,
positions and directions to 1e-6.

A rim is where a tracer's shortcuts meet the reference's closest-surface
rule (AGeoAsphericDisk::ComputeNormal, src/AGeoAsphericDisk.cxx:246-327):
the radial wall and a face are both within rounding of the point.  The
first case below is a ray of the 1e7-ray benchmark batch that lands
1.35e-5 cm inside the secondary's 270 cm rim; a normal choice made in FP32
(where one ulp at 270 cm is 3e-5 cm) read that point as on the rim and
reflected it off the wall instead of the face, and the ray bounced in place
until the point limit.  The offsets stay >= 1e-9 cm from each rim, far
above the 1e-13 cm at which FP64 rounding itself (FMA contraction on the
GPU, none in the oracle) could decide.
"""
import math

import numpy as np
import pytest

import oracle_ref
from robast_gb300 import configs

pytestmark = pytest.mark.gpu

# the benchmark ray (batch index 506682 of schwarzschild_couder(1e7))
REGRESSION_RAY = (-59.547650894990795, -263.3516090739676, 1197.6, 0.0, 0.0, -1.0)
OFFSETS = [s * d for d in (1e-9, 1e-8, 1e-7, 1e-6, 3e-6, 1e-5, 1.35e-5, 2e-5, 5e-5, 1e-4, 1e-3) for s in (1, -1)]
AZIMUTHS = np.linspace(0, 2 * math.pi, 16, endpoint=False) + 0.1


def _rim_batch():
    """Vertical rays from above the secondary (its rim at 270 cm, the
    primary's outer rim at 485 cm), vertical rays from between the mirrors
    (the primary's inner rim at 220 cm, the focal surface's 100 cm and the
    obscuration's 104.3 cm rims), and rays tilted 1 and 4 deg in x aimed at
    points on the secondary's rim."""
    rows = [REGRESSION_RAY]
    for rim, z0 in ((270.0, 1197.6), (485.0, 1197.6), (220.0, 900.0), (100.0, 900.0), (104.3, 900.0)):
        for dr in OFFSETS:
            r = rim + dr
            for ph in AZIMUTHS:
                rows.append((r * math.cos(ph), r * math.sin(ph), z0, 0.0, 0.0, -1.0))
    zs = configs.SC_ZS + 0.5e-4
    for a in (1.0, 4.0):
        d = (math.sin(math.radians(a)), 0.0, -math.cos(math.radians(a)))
        for dr in OFFSETS:
            for ph in AZIMUTHS:
                tx, ty = (270.0 + dr) * math.cos(ph), (270.0 + dr) * math.sin(ph)
                s = 200.0
                rows.append((tx - s * d[0], ty - s * d[1], zs - s * d[2], *d))
    a = np.array(rows)
    n = len(a)
    return {"x": a[:, 0], "y": a[:, 1], "z": a[:, 2], "dx": a[:, 3], "dy": a[:, 4], "dz": a[:, 5],
            "lam": np.full(n, 400e-7), "group": np.zeros(n, dtype=np.int32)}


def _trace(man, batch, precision):
    import torch

    from robast_gb300 import device

    rays = device.to_device(batch, "cuda:0")
    res, st = device.trace(man, rays, precision=precision)
    torch.cuda.synchronize()
    return st, {k: v.cpu().numpy() for k, v in res.items()}


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_rim_rays_match_oracle(precision):
    from robast_gb300 import _native as N

    man, _ = configs.schwarzschild_couder(n_rays=5)
    batch = _rim_batch()
    st, gpu = _trace(man, batch, N.PREC_MIXED if precision == "mixed" else N.PREC_FP64)
    assert st == 0
    ost, ref = oracle_ref.trace(man, configs.to_array(batch), threads=8)
    assert ost == 0
    for k in ("status", "npoints", "last_node"):
        bad = np.nonzero(gpu[k] != ref[k])[0]
        assert bad.size == 0, (k, bad[:10], gpu[k][bad[:10]], ref[k][bad[:10]])
    for k in ("x", "y", "z"):
        err = np.abs(gpu[k] - ref[k]) / np.maximum(1.0, np.abs(ref[k]))
        assert err.max() <= 1e-6, (k, err.max())
    for k in ("dx", "dy", "dz"):
        assert np.abs(gpu[k] - ref[k]).max() <= 1e-6, k
    # the benchmark ray reflects off the secondary's back face and leaves
    assert ref["status"][0] == N.RBG_EXIT and ref["npoints"][0] == 3
    # no ray is left bouncing in place until the point limit
    assert (ref["status"] != N.RBG_SUSPEND).all()
