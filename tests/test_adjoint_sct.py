"""Adjoint gradients through refraction: the Schmidt-Cassegrain batch
(configuration 5: a refracting aspheric corrector plate in front of two
coated mirrors), against central finite differences of the FP64 oracle.

Parameters: per misalignment sample, its secondary's shift in x and y and
rotation about x and y through its vertex.  Every focused ray refracts
twice at the corrector (Snell's transmitted direction, its Sellmeier index
at the ray's wavelength) before its two reflections, so the gradients
exercise the refraction terms of the adjoint.  Losses: the RMS spot radius
and the smoothed 80 % containment radius of each sample, summed, over the
rays whose fate is the same in every trace (the coatings' reflectance
draws can flip a ray between the +h and -h traces).  Agreement to 1e-4 of
the loss change per step, as for the two-mirror telescope.
"""
import numpy as np
import pytest

import oracle_ref
from robast_gb300 import adjoint as A
from robast_gb300 import configs

pytestmark = pytest.mark.gpu

N_SAMPLES = 2
N_RAYS = 24000


def _loss_np(out, stable, group, kind):
    import torch

    tot = 0.0
    for g in range(N_SAMPLES):
        m = stable & (group == g)
        if kind == "rms":
            x, y = out["x"][m], out["y"][m]
            tot += np.sqrt(((x - x.mean()) ** 2 + (y - y.mean()) ** 2).mean())
        else:
            t = lambda v: torch.as_tensor(v, dtype=torch.float64)
            tot += float(A.r80_smooth(t(out["x"]), t(out["y"]), t(m).bool()))
    return tot


@pytest.mark.parametrize("kind", ["rms", "r80"])
def test_sct_gradient_through_refraction(kind):
    import torch

    from robast_gb300 import device

    _, batch = configs.schmidt_cassegrain(n_rays=N_RAYS, n_samples=N_SAMPLES, seed=5)
    arr = configs.to_array(batch)
    group = batch["group"]
    build = A.sct_builder(N_SAMPLES)
    p0 = np.zeros(4 * N_SAMPLES)
    h = A.sct_fd_steps(N_SAMPLES)

    def oracle(p):
        man, _ = build(p)
        st, out = oracle_ref.trace(man, configs.to_array(batch), threads=8)
        assert st == 0
        return out

    # central differences over steps h and h/2, Richardson-extrapolated
    outs = {}
    for k in range(len(p0)):
        for f in (1.0, 0.5):
            for sgn in (1, -1):
                p = p0.copy()
                p[k] += sgn * f * h[k]
                outs[(k, f, sgn)] = oracle(p)
    base = oracle(p0)
    stable = base["status"] == 3
    for o in outs.values():
        stable &= o["status"] == 3
    assert stable.sum() > 8000

    def central(k, f):
        return (_loss_np(outs[(k, f, 1)], stable, group, kind) -
                _loss_np(outs[(k, f, -1)], stable, group, kind)) / (2 * f * h[k])

    fd = np.array([(4 * central(k, 0.5) - central(k, 1.0)) / 3 for k in range(len(p0))])

    rays = device.to_device(batch)
    params = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    TF = A.make_trace_function()
    x, y, focused = TF.apply(params, build, rays)[:3]
    st = torch.as_tensor(stable, device=x.device)
    assert bool((focused[st]).all())
    gd = torch.as_tensor(group, device=x.device)
    loss = 0
    for g in range(N_SAMPLES):
        m = st & (gd == g)
        loss = loss + (A.rms_spot(x, y, m) if kind == "rms" else A.r80_smooth(x, y, m))
    loss.backward()
    grad = params.grad.numpy()
    scale = np.abs(fd * h).max()
    rel = np.abs((grad - fd) * h) / np.maximum(np.abs(fd * h), 1e-3 * scale)
    assert rel.max() < 1e-4, (rel.max(), int(rel.argmax()), grad, fd)
