"""AGeoUtil::ContainmentRadius (src/AGeoUtil.cxx:198-308) on the GPU against
the FP64 oracle's restatement, and the focal-plane histogram it reads.

The device search runs the reference's loop with every SumInRadius probe a
cluster-wide pass; with integer bin counts its sums are exact, so radius
and centre agree with the oracle to rounding (1e-9 relative here).  The
cases: the reference's own testD80 disk (tutorials/unittest_robast.py:
590-610: uniform direction, uniform scale, radius 2 about (1, -1) in a
1000 x 1000 histogram, 80 % containment at 0.8 r0 within 1.5 %), Gaussian
and sparse spots on non-square histograms, an empty histogram, and the
Schwarzschild-Couder focal-plane spots of a real trace.
"""
import numpy as np
import pytest

import oracle_ref
from robast_gb300 import configs

pytestmark = pytest.mark.gpu

RTOL = 1e-9


def _d80_disk(n=2_000_000, seed=3):
    g = np.random.default_rng(seed)
    phi = g.uniform(0, 2 * np.pi, n)
    s = g.uniform(0, 1, n)
    x = 2 * np.cos(phi) * s + 1
    y = 2 * np.sin(phi) * s - 1
    return _hist(x, y, 1000, -3, 3, 1000, -3, 3), (-3, 3, -3, 3)


def _hist(x, y, nx, xlo, xhi, ny, ylo, yhi):
    # TH2D::Fill's bin rule, as the device histogram applies it
    fx = (x - xlo) / (xhi - xlo) * nx
    fy = (y - ylo) / (yhi - ylo) * ny
    ok = (fx >= 0) & (fy >= 0) & (fx < nx) & (fy < ny)
    h = np.zeros((nx, ny))
    np.add.at(h, (fx[ok].astype(np.int64), fy[ok].astype(np.int64)), 1.0)
    return h


def _cases():
    g = np.random.default_rng(11)
    out = []
    out.append(("d80_disk",) + _d80_disk())
    x = g.normal(0.3, 0.05, 300_000)
    y = g.normal(-0.2, 0.08, 300_000)
    out.append(("gauss_500x400", _hist(x, y, 500, 0.0, 0.6, 400, -0.6, 0.2), (0.0, 0.6, -0.6, 0.2)))
    x = g.normal(12.0, 1.0, 600)
    y = g.normal(-3.0, 0.5, 600)
    out.append(("sparse_300x200", _hist(x, y, 300, 7, 17, 200, -6, 0), (7, 17, -6, 0)))
    out.append(("empty", np.zeros((64, 48)), (-1, 1, -1, 1)))
    return out


CASES = _cases()


@pytest.mark.parametrize("name,h,rng", CASES, ids=[c[0] for c in CASES])
def test_containment_radius_matches_oracle(name, h, rng):
    import torch

    from robast_gb300 import device

    xlo, xhi, ylo, yhi = rng
    r_o, x_o, y_o = oracle_ref.containment_radius(h, xlo, xhi, ylo, yhi, 0.8)
    dh = torch.as_tensor(h).cuda()
    r, x, y = device.containment_radius(dh, xlo, xhi, ylo, yhi, 0.8)
    scale = max(abs(xhi - xlo), abs(yhi - ylo))
    assert abs(r - r_o) <= RTOL * max(r_o, 1e-300) + 1e-15 * scale, (r, r_o)
    assert abs(x - x_o) <= RTOL * scale, (x, x_o)
    assert abs(y - y_o) <= RTOL * scale, (y, y_o)
    # the stream-ordered form gives the same numbers, with a zero status
    out = device.containment_radius_async(dh, xlo, xhi, ylo, yhi, 0.8).cpu().numpy()
    assert (out[0], out[1], out[2]) == (r, x, y) and out[3] == 0.0
    if name == "d80_disk":
        # testD80's own bounds
        assert abs(x / 1 - 1) <= 0.015 and abs(y / -1 - 1) <= 0.015 and abs(r / 2 - 0.8) / 0.8 <= 0.015


def test_containment_radius_weighted_counts():
    """Non-integer weights: the sums then depend on the order of addition,
    so a comparison of two sums (sum1 == sum0, sum_x1 > sum1) can go the
    other way on the device and in the oracle, and the two searches part;
    both still stop at the reference's own tolerance (a radius step below
    1e-4 r, so the radii agree to about 1e-4), while the centre is only
    fixed to within the flat top of the containment sum (a shift of 1 % of
    r changes the contained weight by far less than one bin's), so the two
    centres may stop a few hill-climbing steps apart."""
    import torch

    from robast_gb300 import device

    g = np.random.default_rng(4)
    x = g.normal(0.0, 1.0, 200_000)
    y = g.normal(0.5, 0.7, 200_000)
    h = _hist(x, y, 256, -5, 5, 256, -3, 4) * 0.37
    r_o, x_o, y_o = oracle_ref.containment_radius(h, -5, 5, -3, 4, 0.8)
    r, xx, yy = device.containment_radius(torch.as_tensor(h).cuda(), -5, 5, -3, 4, 0.8)
    assert abs(r - r_o) <= 1e-3 * r_o, (r, r_o)
    assert abs(xx - x_o) <= 0.01 * r_o and abs(yy - y_o) <= 0.01 * r_o, (xx, x_o, yy, y_o)


def test_sc_spots_d80_match_oracle():
    """d80 of the Schwarzschild-Couder focal-plane spot of each field angle:
    the GPU histogram of the GPU trace through the GPU search, against the
    oracle's search on the oracle's own focal points binned the same way."""
    import torch

    from robast_gb300 import _native as N
    from robast_gb300 import device

    man, batch = configs.schwarzschild_couder(n_rays=100_000, seed=9)
    rays = device.to_device(batch)
    res, st = device.trace(man, rays, precision=N.PREC_MIXED)
    assert st == 0
    ost, ref = oracle_ref.trace(man, configs.to_array(batch), threads=8)
    assert ost == 0
    group = rays["group"]
    for g in range(int(batch["group"].max()) + 1):
        sel = (ref["status"] == N.RBG_FOCUS) & (batch["group"] == g)
        mx, my = ref["x"][sel].mean(), ref["y"][sel].mean()
        sd = np.sqrt(ref["x"][sel].var() + ref["y"][sel].var())
        hw = 6 * sd
        lims = (mx - hw, mx + hw, my - hw, my + hw)
        h_ref = _hist(ref["x"][sel], ref["y"][sel], 200, lims[0], lims[1], 200, lims[2], lims[3])
        r_o = oracle_ref.containment_radius(h_ref, *lims, 0.8)[0]
        dh = device.focal_histogram(res, 200, lims[0], lims[1], 200, lims[2], lims[3], mask=group == g)
        torch.cuda.synchronize()
        # the same rays land in the same bins (positions agree to ~1e-12)
        np.testing.assert_array_equal(dh.cpu().numpy(), h_ref)
        r = device.containment_radius(dh, *lims, 0.8)[0]
        assert abs(r - r_o) <= RTOL * r_o, (g, r, r_o)
