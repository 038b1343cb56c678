"""Gradients of focal-plane figures of merit through the GPU tracer.

``TraceFunction`` is a ``torch.autograd.Function``: its forward traces a
ray batch (recording each ray's hit points) in a scene built from a
parameter vector, and its backward calls the hand-written adjoint kernel
``rbg_trace_adjoint`` (vector-Jacobian product of the final ray points with
respect to the parameters).  Losses are ordinary torch code on the focal
points, so ``loss.backward()`` gives d loss / d parameters in one forward +
one backward pass -- the gradient step that replaces the Minuit scans of
tutorials/Optimize.C:60-205.

The reference has no gradients.  Effective area (a count of focused rays)
is piecewise constant in the parameters, so its pathwise gradient is zero;
``sc_effective_area`` is a smooth surrogate whose gradient counts the rays
the moving rims sweep across.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Callable, List, Sequence

import numpy as np

from . import _native as N
from . import device

ADJ_ASPH_COEF, ADJ_NODE_SHIFT, ADJ_NODE_ROTATE = 1, 2, 3


class AdjointParam(C.Structure):
    _fields_ = [("kind", C.c_int32), ("node", C.c_int32), ("index", C.c_int32), ("faces", C.c_int32),
                ("pivot", C.c_double * 3)]


def _declare():
    L = N.lib()
    if not getattr(L, "_adj_declared", False):
        L.rbg_trace_adjoint.argtypes = [C.c_void_p, C.c_int64, C.POINTER(N.Result), C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(AdjointParam),
                                        C.c_void_p, C.POINTER(C.c_int64), C.c_void_p]
        L._adj_declared = True
    return L


@dataclass
class ParamSpec:
    """One differentiable parameter: kind, physical node id, index (K_j or
    axis), face mask for coefficients, pivot for rotations."""
    kind: int
    node: int
    index: int
    faces: int = 3
    pivot: Sequence[float] = (0.0, 0.0, 0.0)

    def as_c(self):
        return AdjointParam(self.kind, self.node, self.index, self.faces, (C.c_double * 3)(*self.pivot))


def trace_with_history(manager, rays, precision=N.PREC_MIXED, history=8, stream=None):
    n = rays["x"].numel()
    res = device.alloc_result(n, rays["x"].device, history)
    res, st = device.trace(manager, rays, res, precision=precision, stream=stream)
    return res, st


def vjp(manager, res, specs: List[ParamSpec], gx, gy, gz=None, stream=None, lam=None, gpts=None):
    """dL/dp for cotangents (gx, gy, gz) of the final points and gpts
    (n, hist_cap, 3) of the recorded points (device tensors, None = 0);
    lam: the rays' wavelengths (needed by scenes with lenses)."""
    import torch

    L = _declare()
    n = res["x"].numel()
    rr = device._result_struct(res)
    arr = (AdjointParam * max(1, len(specs)))(*[s.as_c() for s in specs])
    out = torch.zeros(len(specs), dtype=torch.float64, device=res["x"].device)
    skipped = C.c_int64(0)
    st = (stream if stream is not None else torch.cuda.current_stream()).cuda_stream
    gp = gpts.contiguous() if gpts is not None else None
    N.check(L.rbg_trace_adjoint(manager.scene.handle, n, C.byref(rr), device._ptr(lam), device._ptr(gx),
                                device._ptr(gy), device._ptr(gz), device._ptr(gp), len(specs), arr,
                                device._ptr(out), C.byref(skipped), C.c_void_p(st)), "rbg_trace_adjoint")
    return out, skipped.value


def make_trace_function():
    import torch

    class TraceFunction(torch.autograd.Function):
        """forward(params, build, rays, precision, history) ->
        (x, y, focused, points, nodes).

        ``build(params_numpy) -> (manager, [ParamSpec])`` constructs the
        scene at the given parameter values.  points (n, history, 3) are
        the recorded hit points (differentiable at reflections,
        refractions and the end point), nodes (n, history) their nodes."""

        last_skipped = 0  # rays the last backward pass could not differentiate

        @staticmethod
        def forward(ctx, params, build: Callable, rays, precision=N.PREC_MIXED, history=8):
            man, specs = build(params.detach().cpu().numpy())
            res, st = trace_with_history(man, rays, precision, history)
            if st not in (N.RBG_OK,):
                N.check(st, "rbg_trace")
            focused = res["status"] == N.RBG_FOCUS
            ctx.man, ctx.specs, ctx.res, ctx.lam = man, specs, res, rays["lam"]
            ctx.param_device, ctx.param_dtype = params.device, params.dtype
            nodes = res["hist_node"].clone()
            ctx.mark_non_differentiable(focused, nodes)
            # outputs the loss does not use get no (zero-filled) cotangent
            ctx.set_materialize_grads(False)
            return res["x"].clone(), res["y"].clone(), focused, res["hist_xyzt"][..., :3].clone(), nodes

        @staticmethod
        def backward(ctx, gx, gy, _gf, gp, _gn):
            gx = gx.contiguous() if gx is not None else None
            gy = gy.contiguous() if gy is not None else None
            if gx is None and gy is None and gp is None:
                ctx.skipped = 0
                z = torch.zeros(len(ctx.specs), dtype=ctx.param_dtype, device=ctx.param_device)
                return z, None, None, None, None
            g, skipped = vjp(ctx.man, ctx.res, ctx.specs, gx, gy, lam=ctx.lam, gpts=gp)
            ctx.skipped = TraceFunction.last_skipped = skipped
            return g.to(device=ctx.param_device, dtype=ctx.param_dtype), None, None, None, None

    return TraceFunction


def rms_spot(x, y, mask):
    """RMS spot radius of the rays of `mask`: sqrt(<|p - <p>|^2>).  Masked
    arithmetic rather than boolean indexing: no host synchronisation, and
    the backward pass is elementwise."""
    import torch

    w = mask.to(x.dtype)
    n = w.sum()
    xm = torch.where(mask, x, torch.zeros_like(x))
    ym = torch.where(mask, y, torch.zeros_like(y))
    mx, my = xm.sum() / n, ym.sum() / n
    return ((w * ((xm - mx) ** 2 + (ym - my) ** 2)).sum() / n).sqrt()


def rms_spot_groups(x, y, mask, group, n_groups):
    """Sum over groups g < n_groups of the RMS spot radius of the rays of
    `mask` in group g (each group's radius as rms_spot).  Two passes of
    rbg_focal_moments: every group's count and centroid, then the sums of
    squares about the centroids (no cancellation between <x^2> and
    <x>^2); the backward pass is one elementwise expression,
    d r_g / d x_i = (x_i - <x>_g) / (n_g r_g)."""
    import torch

    from . import device

    class _RmsGroups(torch.autograd.Function):
        @staticmethod
        def forward(ctx, xx, yy):
            status = torch.where(mask, torch.full_like(mask, N.RBG_FOCUS, dtype=torch.uint8),
                                 torch.zeros_like(mask, dtype=torch.uint8))
            m = device.focal_moments({"status": status, "x": xx, "y": yy, "t": None}, group, n_groups)
            n = m[:, 0].clamp(min=1.0)
            g = group.long()
            mx, my = m[:, 1] / n, m[:, 2] / n
            d = device.focal_moments({"status": status, "x": xx - mx[g], "y": yy - my[g], "t": None}, group,
                                     n_groups)
            ex, ey = d[:, 1] / n, d[:, 2] / n  # the first pass's centroid error
            mx, my = mx + ex, my + ey
            r = ((d[:, 3] + d[:, 4]) / n - ex * ex - ey * ey).clamp(min=0.0).sqrt()
            ctx.save_for_backward(xx, yy, mx, my, n, r)
            return r[m[:, 0] > 0].sum()

        @staticmethod
        def backward(ctx, go):
            xx, yy, mx, my, n, r = ctx.saved_tensors
            g = group.long()
            k = torch.where(r > 0, go / (n * r), torch.zeros_like(r))
            kg = torch.where(mask, k[g], torch.zeros_like(xx))
            return kg * (xx - mx[g]), kg * (yy - my[g])

    return _RmsGroups.apply(x, y)


def r80_smooth(x, y, mask, width_frac=0.05, fraction=0.8):
    """Differentiable 80 % containment radius about the centroid: the root r
    of G(r) = <sigmoid((r - rho_i) / (w r))> - fraction = 0 with w =
    width_frac (the sigmoid's width scales with r itself, so G is smooth in
    the ray positions and strictly increasing in r).  The root is found by
    bisection without gradient; one implicit-function step
    r0 - G(r0) / G'(r0), with G'(r0) = <s (1 - s) rho_i / (w r0^2)> held
    fixed, carries dr/dx = -(dG/dx) / G'(r)."""
    import torch

    xs, ys = x[mask], y[mask]
    cx, cy = xs.mean(), ys.mean()
    rho = torch.sqrt((xs - cx) ** 2 + (ys - cy) ** 2 + 1e-30)
    with torch.no_grad():
        lo, hi = torch.zeros_like(rho[0]), 2 * rho.max() + 1e-30
        for _ in range(100):
            mid = 0.5 * (lo + hi)
            g = torch.sigmoid((mid - rho) / (width_frac * mid)).mean()
            lo, hi = torch.where(g < fraction, mid, lo), torch.where(g < fraction, hi, mid)
        r0 = 0.5 * (lo + hi)
        s = torch.sigmoid((r0 - rho) / (width_frac * r0))
        dG = (s * (1 - s) * rho).mean() / (width_frac * r0 * r0)
    G = torch.sigmoid((r0 - rho) / (width_frac * r0)).mean() - fraction
    return r0 - G / dG


# ---------------------------------------------------------------------------
# Schwarzschild-Couder parameterisation: 8 + 8 aspheric coefficients and
# the secondary's shift (3) and rotation (3) about its vertex
# ---------------------------------------------------------------------------
def sc_parameters(primary_k=None, secondary_k=None):
    from .configs import SC_PRIMARY_K, SC_SECONDARY_K

    kp = np.array(SC_PRIMARY_K if primary_k is None else primary_k, dtype=float)
    ks = np.array(SC_SECONDARY_K if secondary_k is None else secondary_k, dtype=float)
    return np.concatenate([kp, ks, np.zeros(6)])


def sc_builder(n_rays=0):
    """build(params) for the Schwarzschild-Couder telescope of configs.py."""
    from .configs import SC_ZS, schwarzschild_couder

    def build(p):
        man, _ = schwarzschild_couder(n_rays=5, primary_k=p[0:8], secondary_k=p[8:16], perturb=0.0,
                                      secondary_shift=tuple(p[16:19]), secondary_tilt=tuple(p[19:22]))
        names = man.scene.node_names()
        prim = names.index("primaryMirror")
        sec = names.index("secondaryMirror")
        specs = [ParamSpec(ADJ_ASPH_COEF, prim, j, 3) for j in range(8)]
        specs += [ParamSpec(ADJ_ASPH_COEF, sec, j, 3) for j in range(8)]
        specs += [ParamSpec(ADJ_NODE_SHIFT, sec, a) for a in range(3)]
        pivot = (float(p[16]), float(p[17]), SC_ZS + float(p[18]))
        specs += [ParamSpec(ADJ_NODE_ROTATE, sec, a, pivot=pivot) for a in range(3)]
        return man, specs

    return build


def fd_steps(params):
    """Central-difference steps: coefficient steps that move the sag by
    ~1e-5 cm at r = 4.85 m, 1e-4 cm shifts, 1e-6 rad rotations."""
    h = np.empty_like(params)
    for j in range(8):
        h[j] = h[8 + j] = 1e-5 / (485.0 ** (2 * (j + 1)))
    h[16:19] = 1e-4
    h[19:22] = 1e-6
    return h


# ---------------------------------------------------------------------------
# Schmidt-Cassegrain batch (configuration 5): per misalignment sample, the
# secondary's shift in x and y and rotation about x and y (through its
# displaced vertex), as increments on top of the drawn misalignment
# ---------------------------------------------------------------------------
def sct_builder(n_samples: int, seed: int = 5):
    """build(params) for configs.schmidt_cassegrain with 4 parameters per
    sample (shift x, shift y, rotation x, rotation y of its secondary)."""
    from .configs import schmidt_cassegrain

    def build(p):
        inc = np.asarray(p, dtype=float).reshape(n_samples, 4)
        man, _ = schmidt_cassegrain(n_rays=n_samples, n_samples=n_samples, seed=seed, increments=inc)
        names = man.scene.node_names()
        flat = man.scene.flat
        specs = []
        for v in range(n_samples):
            k = names.index(f"secondary{v}")
            # the rotation pivot: the node's vertex (local (0, 0, zs)) in the world
            sdisk = man.scene.builder.volume_objs[flat.nodes[k].volume].shape
            zs = max(sdisk.z1, sdisk.z2)
            m = np.array(flat.nodes[k].m[:])
            pivot = tuple(m[:9].reshape(3, 3) @ np.array([0.0, 0.0, zs]) + m[9:])
            specs += [ParamSpec(ADJ_NODE_SHIFT, k, a) for a in range(2)]
            specs += [ParamSpec(ADJ_NODE_ROTATE, k, a, pivot=pivot) for a in range(2)]
        return man, specs

    return build


def sct_fd_steps(n_samples: int):
    """Central-difference steps: 1e-4 cm shifts, 1e-6 rad rotations."""
    return np.tile([1e-4, 1e-4, 1e-6, 1e-6], n_samples)


# ---------------------------------------------------------------------------
# Effective area: a smooth surrogate with a pathwise gradient
# ---------------------------------------------------------------------------
def _rot_zyx(t):
    """Rz(t[2]) Ry(t[1]) Rx(t[0]) (TGeoRotation's RotateX, then RotateY,
    then RotateZ; radians) as a torch matrix."""
    import torch

    cx, sx = torch.cos(t[0]), torch.sin(t[0])
    cy, sy = torch.cos(t[1]), torch.sin(t[1])
    cz, sz = torch.cos(t[2]), torch.sin(t[2])
    one, zero = torch.ones_like(cx), torch.zeros_like(cx)
    rx = torch.stack([torch.stack([one, zero, zero]), torch.stack([zero, cx, -sx]), torch.stack([zero, sx, cx])])
    ry = torch.stack([torch.stack([cy, zero, sy]), torch.stack([zero, one, zero]), torch.stack([-sy, zero, cy])])
    rz = torch.stack([torch.stack([cz, -sz, zero]), torch.stack([sz, cz, zero]), torch.stack([zero, zero, one])])
    return rz @ ry @ rx


def sc_effective_area(params, pts, nodes, o, d, keep, area_per_ray, node_ids, width=1.0):
    """Effective area of the Schwarzschild-Couder telescope (the focused
    count times the area per ray, tutorials/SchwarzschildCouder.C:139) as a
    smooth function of the parameters.  A focused ray passed five rims: it
    missed the secondary on its way down (outside its 270 cm rim), hit the
    primary between its 220 and 485 cm rims, hit the secondary inside its
    rim and the focal surface inside its 100 cm rim.  Its weight is the
    product of tanh(margin / width) over those margins, so
    Aeff_s = area_per_ray * sum_i w_i over the rays of `keep` (focused).
    The margins at the hit points carry the hit points' gradient (the
    adjoint, through `pts`); the secondary's rim also moves with its shift
    and tilt (params[16:22]) explicitly.  As width -> 0 the gradient counts
    the rays a moving rim sweeps across (tanh' integrates to 1 over m > 0),
    the derivative of the focused count the pathwise gradient cannot see.

    pts, nodes: the recorded points and nodes (TraceFunction outputs); o, d:
    the rays' start points and directions (n, 3); node_ids: physical node
    ids of "primary", "secondary" and "focal"."""
    import torch

    from .configs import SC_ZS

    R = _rot_zyx(params[19:22])
    c = torch.tensor([0.0, 0.0, SC_ZS], dtype=params.dtype, device=params.device)
    t = c - R @ c + params[16:19]
    o_k, d_k = o[keep], d[keep]
    P, Nn = pts[keep], nodes[keep]

    def local_sec(v, direction=False):
        return (v if direction else v - t) @ R  # R^T (v - t) for row vectors

    # the secondary's rim height (its upper face at r = 270 cm)
    ks = params[8:16]
    r2 = 270.0 ** 2
    z_rim = SC_ZS + 1e-4 + sum(ks[j] * r2 ** (j + 1) for j in range(8))
    ol, dl = local_sec(o_k), local_sec(d_k, True)
    s = (z_rim - ol[:, 2]) / dl[:, 2]
    q = ol + s[:, None] * dl
    m_shadow = torch.sqrt(q[:, 0] ** 2 + q[:, 1] ** 2) - 270.0

    def at(node):
        sel = (Nn == node).to(P.dtype)
        return (P * sel[..., None]).sum(dim=1)  # the (one) recorded point on that node

    pp = at(node_ids["primary"])
    rp = torch.sqrt(pp[:, 0] ** 2 + pp[:, 1] ** 2)
    ps = local_sec(at(node_ids["secondary"]))
    rs = torch.sqrt(ps[:, 0] ** 2 + ps[:, 1] ** 2)
    pf = at(node_ids["focal"])
    rf = torch.sqrt(pf[:, 0] ** 2 + pf[:, 1] ** 2)
    margins = [m_shadow, 485.0 - rp, rp - 220.0, 270.0 - rs, 100.0 - rf]
    w = torch.ones_like(rp)
    for m in margins:
        w = w * torch.tanh(torch.clamp(m, min=0.0) / width)
    return area_per_ray * w.sum()
