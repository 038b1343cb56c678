"""Gradient-driven optical design.

tutorials/Optimize.C:60-205 fits a design with Minuit2, tracing the whole
ray batch at every function call (and twice per parameter for each
numerical gradient).  Here a design step is one forward trace that keeps
the hit records plus one adjoint pass (rbg_trace_adjoint) through
torch.autograd, so any torch optimiser takes gradient steps on the
parameters a scene builder exposes (aspheric coefficients, rigid motions of
nodes).  Parameters are optimised in normalised units u = (p - p0) / scale,
since their natural magnitudes span dozens of decades (8-term aspheric
coefficients).
"""
from __future__ import annotations

from typing import Callable, List, Optional, Sequence

import numpy as np

from . import adjoint as A


class DesignOptimizer:
    """Minimise loss(x, y, focused) over the focal-plane points of `rays`
    traced through build(params).

    build(params_numpy) -> (manager, [ParamSpec]) as for
    adjoint.make_trace_function; loss maps device tensors (x, y, focused
    mask) to a scalar tensor (adjoint.rms_spot, adjoint.r80_smooth, ...).
    """

    def __init__(self, build: Callable, params0: Sequence[float], rays, loss: Optional[Callable] = None,
                 scale: Optional[Sequence[float]] = None, optimizer=None, lr: float = 0.05, **opt_kwargs):
        import torch

        self.build = build
        self.rays = rays
        self.p0 = np.asarray(params0, dtype=float)
        self.scale = np.asarray(scale if scale is not None else np.maximum(np.abs(self.p0), 1e-12), dtype=float)
        self.loss_fn = loss if loss is not None else (lambda x, y, f: A.rms_spot(x, y, f))
        self.u = torch.zeros(len(self.p0), dtype=torch.float64, requires_grad=True)
        opt = optimizer if optimizer is not None else torch.optim.Adam
        self.opt = opt([self.u], lr=lr, **opt_kwargs)
        self._p0 = torch.tensor(self.p0, dtype=torch.float64)
        self._scale = torch.tensor(self.scale, dtype=torch.float64)
        self.TF = A.make_trace_function()
        self.history: List[float] = []
        self.traces = 0

    @property
    def params(self) -> np.ndarray:
        return self.p0 + self.scale * self.u.detach().cpu().numpy()

    def evaluate(self):
        """Loss at the current parameters (a forward trace only)."""
        import torch

        with torch.no_grad():
            p = self._p0 + self._scale * self.u
            x, y, f = self.TF.apply(p, self.build, self.rays)[:3]
            self.traces += 1
            return float(self.loss_fn(x, y, f))

    def step(self) -> float:
        """One gradient step: forward trace with hit records, adjoint pass,
        optimiser update.  Returns the loss before the update."""
        self.opt.zero_grad()
        p = self._p0 + self._scale * self.u
        x, y, f = self.TF.apply(p, self.build, self.rays)[:3]
        loss = self.loss_fn(x, y, f)
        loss.backward()
        self.traces += 2
        self.opt.step()
        v = float(loss.detach())
        self.history.append(v)
        return v

    def run(self, steps: int) -> List[float]:
        for _ in range(steps):
            self.step()
        return self.history
