"""Gradient-driven design (tutorials/Optimize.C, with gradient steps in
place of Minuit scans): recover a misaligned Schwarzschild-Couder secondary
from its RMS spot alone."""
import numpy as np
import pytest

from robast_gb300 import adjoint as A
from robast_gb300 import configs

pytestmark = pytest.mark.gpu


def test_secondary_alignment_recovered_by_gradient_steps():
    import torch

    from robast_gb300 import device
    from robast_gb300.optimize import DesignOptimizer

    _, batch = configs.schwarzschild_couder(n_rays=20000, angles=(0.0,), seed=31)
    rays = device.to_device(batch)
    p_true = A.sc_parameters()
    build_full = A.sc_builder()
    # optimise the secondary's 3 shifts and 3 tilts; the coefficients stay
    misalign = np.array([0.3, -0.2, 0.5, 4e-4, -3e-4, 0.0])

    def build(u6):
        p = p_true.copy()
        p[16:22] = u6
        man, specs = build_full(p)
        return man, specs[16:22]

    opt = DesignOptimizer(build, misalign, rays, scale=[0.1, 0.1, 0.1, 1e-4, 1e-4, 1e-4], lr=0.2)
    start = opt.evaluate()
    opt.run(60)
    end = opt.evaluate()
    best = min(opt.history)
    torch.cuda.synchronize()
    # the spot at the true alignment, for scale
    x0, y0, f0 = opt.TF.apply(torch.zeros(6, dtype=torch.float64), build, rays)[:3]
    nominal = float(A.rms_spot(x0, y0, f0))
    # most of the excess spot size over the aligned design is removed (a
    # lateral shift and a tilt partly compensate each other, so the
    # parameters themselves need not return to zero)
    assert min(best, end) < nominal + 0.3 * (start - nominal), (start, end, best, nominal)
    assert end < start
    # two traces per gradient step, against 2 x 6 + 1 for a central-difference step
    assert opt.traces == 2 * 60 + 2
