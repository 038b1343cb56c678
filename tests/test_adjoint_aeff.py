"""Gradient of the smooth effective-area surrogate of the Schwarzschild-
Couder telescope (adjoint.sc_effective_area): the margins of each focused
ray to the five rims it passed, through the adjoint's hit-point gradients
(the cotangents of recorded points) and the secondary rim's own motion,
against central differences of the same surrogate on the FP64 oracle's
recorded points.  Agreement to 1e-4 of the loss change per step over the
16 aspheric coefficients and the secondary's 6 rigid degrees of freedom.
"""
import numpy as np
import pytest

import oracle_ref
from robast_gb300 import adjoint as A
from robast_gb300 import configs

pytestmark = pytest.mark.gpu

N_RAYS = 30000
WIDTH = 1.0


def _ids(man):
    names = man.scene.node_names()
    return {"primary": names.index("primaryMirror"), "secondary": names.index("secondaryMirror"),
            "focal": names.index("focalPlane")}


def _surrogate_np(build, p, batch, stable, area):
    import torch

    man, _ = build(p)
    st, out = oracle_ref.trace(man, configs.to_array(batch), threads=8, history=8)
    assert st == 0
    t = lambda v: torch.as_tensor(np.ascontiguousarray(v))
    pts = t(out["hist_xyzt"].reshape(len(batch["x"]), 8, 4)[..., :3])
    nodes = t(out["hist_node"].reshape(len(batch["x"]), 8))
    o = t(np.stack([batch["x"], batch["y"], batch["z"]], axis=1))
    d = t(np.stack([batch["dx"], batch["dy"], batch["dz"]], axis=1))
    foc = out["status"] == 3
    val = A.sc_effective_area(torch.as_tensor(p, dtype=torch.float64), pts, nodes, o, d, t(stable), area,
                              _ids(man), WIDTH)
    return float(val), foc


def test_effective_area_gradient():
    import torch

    from robast_gb300 import device

    _, batch = configs.schwarzschild_couder(n_rays=N_RAYS, angles=(0.0, 3.0), seed=31)
    n = len(batch["x"])
    area = np.pi * 500.0 ** 2 / (n / 2)
    build = A.sc_builder()
    p0 = A.sc_parameters()
    h = A.fd_steps(p0)
    everything = np.ones(n, dtype=bool)
    _, stable = _surrogate_np(build, p0, batch, everything, area)
    for k in range(len(p0)):
        for f in (1.0, 0.5):
            for sgn in (1, -1):
                p = p0.copy()
                p[k] += sgn * f * h[k]
                _, foc = _surrogate_np(build, p, batch, everything, area)
                stable &= foc
    assert stable.sum() > 10000

    def central(k, f):
        pp, pm = p0.copy(), p0.copy()
        pp[k] += f * h[k]
        pm[k] -= f * h[k]
        return (_surrogate_np(build, pp, batch, stable, area)[0] -
                _surrogate_np(build, pm, batch, stable, area)[0]) / (2 * f * h[k])

    fd = np.array([(4 * central(k, 0.5) - central(k, 1.0)) / 3 for k in range(len(p0))])

    rays = device.to_device(batch)
    params = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    TF = A.make_trace_function()
    x, y, focused, pts, nodes = TF.apply(params, build, rays)
    keep = torch.as_tensor(stable, device=x.device)
    assert bool(focused[keep].all())
    o = torch.stack([rays["x"], rays["y"], rays["z"]], dim=1)
    d = torch.stack([rays["dx"], rays["dy"], rays["dz"]], dim=1)
    man, _ = build(p0)
    ids = _ids(man)
    pdev = params.to(x.device) if params.device != x.device else params
    aeff = A.sc_effective_area(pdev, pts, nodes, o, d, keep, area, ids, WIDTH)
    aeff.backward()
    assert TF.last_skipped == 0
    g = params.grad.numpy()
    scale = np.abs(fd * h).max()
    rel = np.abs((g - fd) * h) / np.maximum(np.abs(fd * h), 1e-3 * scale)
    assert rel.max() < 1e-4, (rel.max(), int(rel.argmax()), g, fd)
    # the surrogate is close to the count it smooths
    assert abs(float(aeff) / (area * float(keep.sum())) - 1) < 0.05
