"""Adjoint gradients vs central finite differences of the FP64 oracle.

The loss is the RMS spot radius (and the smoothed 80 % containment radius)
of the on-axis Schwarzschild-Couder PSF as a function of the 16 aspheric
coefficients and the secondary's 6 rigid degrees of freedom.  The GPU
adjoint (one forward with hit records + one backward) must agree with
central differences of the oracle's FP64 trace to 1e-4 relative.
"""
import numpy as np
import pytest

import oracle_ref
from robast_gb300 import adjoint as A
from robast_gb300 import configs

pytestmark = pytest.mark.gpu

N_RAYS = 20000


def _batch():
    _, batch = configs.schwarzschild_couder(n_rays=N_RAYS, angles=(0.0,), seed=21)
    return batch


def _oracle_points(build, params, arr):
    man, _ = build(params)
    st, out = oracle_ref.trace(man, arr, threads=8)
    assert st == 0
    return out


def _loss_np(out, mask, kind):
    x, y = out["x"][mask], out["y"][mask]
    if kind == "rms":
        return np.sqrt(((x - x.mean()) ** 2 + (y - y.mean()) ** 2).mean())
    import torch

    t = lambda v: torch.as_tensor(v, dtype=torch.float64)
    return float(A.r80_smooth(t(out["x"]), t(out["y"]), t(mask).bool()))


@pytest.mark.parametrize("kind", ["rms", "r80"])
def test_sc_gradient_vs_finite_differences(kind):
    import torch

    from robast_gb300 import device

    batch = _batch()
    arr = configs.to_array(batch)
    build = A.sc_builder()
    p0 = A.sc_parameters()
    base = _oracle_points(build, p0, arr)
    mask = base["status"] == 3
    assert mask.sum() > 3000

    # adjoint on the GPU (mixed-precision forward with hit records)
    rays = device.to_device(batch)
    params = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    TF = A.make_trace_function()
    x, y, focused = TF.apply(params, build, rays)[:3]
    m = torch.as_tensor(mask, device=x.device)
    assert bool((focused == m).all())
    loss = A.rms_spot(x, y, m) if kind == "rms" else A.r80_smooth(x, y, m)
    loss.backward()
    g = params.grad.numpy()

    # central differences of the oracle, same rays and mask, Richardson-
    # extrapolated over steps h and h/2: (4 D(h/2) - D(h)) / 3 cancels the
    # O(h^2) truncation term.  That term matters for the smoothed r80, whose
    # sigmoid is only ~5 % of r80 wide: a 1 urad secondary tilt moves the
    # spot by a tenth of that width, and plain D(h) is then off by ~5e-4.
    h = A.fd_steps(p0)
    fd = np.zeros_like(p0)

    def central(k, step):
        pp, pm = p0.copy(), p0.copy()
        pp[k] += step
        pm[k] -= step
        op, om = _oracle_points(build, pp, arr), _oracle_points(build, pm, arr)
        assert ((op["status"] == 3) == mask).all() and ((om["status"] == 3) == mask).all()
        return (_loss_np(op, mask, kind) - _loss_np(om, mask, kind)) / (2 * step)

    for k in range(len(p0)):
        fd[k] = (4 * central(k, 0.5 * h[k]) - central(k, h[k])) / 3
    # compare in units of the step (the loss change per step)
    scale = np.abs(fd * h).max()
    err = np.abs((g - fd) * h)
    rel = err / np.maximum(np.abs(fd * h), 1e-3 * scale)
    assert rel.max() < 1e-4, (rel.max(), int(rel.argmax()), g, fd)


def test_rms_spot_groups_matches_per_group():
    """The grouped RMS loss (two moment passes on the device, elementwise
    backward) equals the sum of the per-group losses and their gradients."""
    import torch

    g = torch.Generator().manual_seed(4)
    n, groups = 200_000, 5
    x = (30 * torch.rand(n, generator=g, dtype=torch.float64) + 0.2 * torch.randn(n, generator=g,
                                                                                  dtype=torch.float64)).cuda()
    y = (0.2 * torch.randn(n, generator=g, dtype=torch.float64)).cuda()
    group = (torch.arange(n) * groups // n).to(torch.int32).cuda()
    mask = (torch.rand(n, generator=g) < 0.6).cuda()
    xa, ya = x.clone().requires_grad_(), y.clone().requires_grad_()
    la = A.rms_spot_groups(xa, ya, mask, group, groups)
    la.backward()
    xb, yb = x.clone().requires_grad_(), y.clone().requires_grad_()
    lb = sum(A.rms_spot(xb, yb, mask & (group == k)) for k in range(groups))
    lb.backward()
    assert abs(float(la) - float(lb)) <= 1e-12 * abs(float(lb))
    for a, b in ((xa.grad, xb.grad), (ya.grad, yb.grad)):
        assert float((a - b).abs().max()) <= 1e-12 * float(b.abs().max())
