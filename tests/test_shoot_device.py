"""ARayShooter sources generated on the GPU (rbg_shoot_device) against the
host generators (rbg_shoot): the same Philox draws per ray, positions and
directions bit for bit for the circle / cone / rectangle sources and the
grids, to 1e-15 for the sphere sources (device cos / sin / acos)."""
import numpy as np
import pytest

import robast_gb300 as R
from robast_gb300 import _native as N

pytestmark = pytest.mark.gpu

ROT = R.TGeoRotation("", 20.0, 35.0, -10.0)
TR = R.TGeoTranslation(1.5, -2.0, 300.0)
CASES = [
    ("random_circle", N.RBG_SHOOT_RANDOM_CIRCLE, [110.0], 20000, True),
    ("random_cone", N.RBG_SHOOT_RANDOM_CONE, [5.0, 100.0], 20000, True),
    ("random_rectangle", N.RBG_SHOOT_RANDOM_RECTANGLE, [40.0, 20.0], 20000, True),
    ("rectangle", N.RBG_SHOOT_RECTANGLE, [40.0, 20.0, 37, 23], 0, True),
    ("circle", N.RBG_SHOOT_CIRCLE, [50.0, 12, 7], 0, False),
    ("random_sphere", N.RBG_SHOOT_RANDOM_SPHERE, [], 20000, False),
    ("random_spherical_cone", N.RBG_SHOOT_RANDOM_SPHERICAL_CONE, [12.0], 20000, False),
]


@pytest.mark.parametrize("name,kind,params,n,exact", CASES, ids=[c[0] for c in CASES])
def test_device_source_matches_host(name, kind, params, n, exact):
    import torch

    from robast_gb300 import device
    from robast_gb300.manager import ARayShooter

    v = (0.1, -0.2, -1.0)
    if kind == N.RBG_SHOOT_CIRCLE:
        cnt = 1 + params[2] * params[1] * (params[1] + 1) // 2
    elif kind == N.RBG_SHOOT_RECTANGLE:
        cnt = params[2] * params[3]
    else:
        cnt = n
    host = ARayShooter._shoot(kind, params, cnt, 400e-7, ROT, TR, v, seed=99, first_id=5)
    dev = device.shoot(kind, params, cnt, 400e-7, ROT, TR, v, seed=99, first_id=5)
    torch.cuda.synchronize()
    assert dev["x"].numel() == len(host.x) == cnt
    for f, hf in (("x", "x"), ("y", "y"), ("z", "z"), ("dx", "dx"), ("dy", "dy"), ("dz", "dz"), ("lam", "lam")):
        got = dev[f].cpu().numpy()
        want = getattr(host, hf)
        if exact:
            np.testing.assert_array_equal(got, want, err_msg=f)
        else:
            np.testing.assert_allclose(got, want, rtol=0, atol=1e-13 * max(1.0, np.abs(want).max()), err_msg=f)
