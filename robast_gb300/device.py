"""Device-resident tracing: ray batches held as CUDA tensors.

PyTorch provides device memory and streams only; all work is done by the
library's kernels through the C ABI (rbg_trace, rbg_focal_moments,
rbg_focal_histogram, rbg_containment_radius).
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional

import numpy as np

from . import _native as N

RAY_FIELDS = ("x", "y", "z", "t", "dx", "dy", "dz", "lam")
OUT_F64 = ("x", "y", "z", "t", "dx", "dy", "dz")


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("no CUDA device: the tracer has no CPU path")
    return torch


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def to_device(batch: Dict[str, np.ndarray], device="cuda:0") -> Dict[str, "object"]:
    torch = _torch()
    out = {}
    n = len(batch["x"])
    for f in RAY_FIELDS:
        src = batch.get(f)
        if src is None:
            src = np.zeros(n)
        out[f] = torch.as_tensor(np.ascontiguousarray(src, dtype=np.float64)).to(device)
    if "group" in batch:
        out["group"] = torch.as_tensor(np.ascontiguousarray(batch["group"], dtype=np.int32)).to(device)
    return out


def alloc_result(n: int, device="cuda:0", history: int = 0):
    torch = _torch()
    res = {f: torch.empty(n, dtype=torch.float64, device=device) for f in OUT_F64}
    res["status"] = torch.empty(n, dtype=torch.uint8, device=device)
    res["npoints"] = torch.empty(n, dtype=torch.int32, device=device)
    res["last_node"] = torch.empty(n, dtype=torch.int32, device=device)
    if history:
        res["hist_xyzt"] = torch.empty((n, history, 4), dtype=torch.float64, device=device)
        res["hist_node"] = torch.empty((n, history), dtype=torch.int32, device=device)
    return res


def _rays_struct(rays) -> N.Rays:
    dp = C.POINTER(C.c_double)
    n = rays["x"].numel()
    ptrs = [C.cast(C.c_void_p(rays[f].data_ptr()), dp) for f in RAY_FIELDS]
    return N.Rays(n, *ptrs)


def _result_struct(res) -> N.Result:
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int32)
    r = N.Result()
    r.status = C.cast(C.c_void_p(res["status"].data_ptr()), C.POINTER(C.c_uint8)) if "status" in res else None
    r.npoints = C.cast(C.c_void_p(res["npoints"].data_ptr()), ip) if "npoints" in res else None
    r.last_node = C.cast(C.c_void_p(res["last_node"].data_ptr()), ip) if "last_node" in res else None
    for f in OUT_F64:
        setattr(r, f, C.cast(C.c_void_p(res[f].data_ptr()), dp) if f in res else None)
    if "hist_xyzt" in res:
        r.hist_cap = res["hist_xyzt"].shape[1]
        r.hist_xyzt = C.cast(C.c_void_p(res["hist_xyzt"].data_ptr()), dp)
        r.hist_node = C.cast(C.c_void_p(res["hist_node"].data_ptr()), ip)
    else:
        r.hist_cap = 0
    return r


# per-device take-up order workspace shared by every scene this process
# traces (allocated by torch, handed to rbg_trace in its options)
_WORKSPACE = {}


def workspace(n: int, device):
    """A device buffer of at least rbg_trace_workspace_bytes(n) bytes,
    grown on demand and kept for later traces on `device`."""
    torch = _torch()
    need = int(N.lib().rbg_trace_workspace_bytes(int(n)))
    if need == 0:
        return None
    dev = torch.device(device)
    ws = _WORKSPACE.get(dev)
    if ws is None or ws.numel() < need:
        _WORKSPACE.pop(dev, None)
        ws = torch.empty(need, dtype=torch.uint8, device=dev)
        _WORKSPACE[dev] = ws
    return ws


def trace(manager, rays, res=None, precision: Optional[int] = None, stream=None, check: bool = True,
          workspace_buf="auto"):
    """AOpticsManager::TraceNonSequential on device tensors; returns the
    result dict and the C status.  workspace_buf: "auto" (this module's
    shared buffer), None (the scene's own, rbg_scene_reserve) or a uint8
    device tensor for the take-up order."""
    torch = _torch()
    scene = manager._ensure_scene()
    n = rays["x"].numel()
    if res is None:
        res = alloc_result(n, rays["x"].device)
    rs = _rays_struct(rays)
    rr = _result_struct(res)
    opts = manager.trace_options(precision)
    ws = workspace(n, rays["x"].device) if isinstance(workspace_buf, str) else workspace_buf
    if ws is not None:
        opts.workspace = ws.data_ptr()
        opts.workspace_bytes = ws.numel()
    st_ptr = (stream if stream is not None else torch.cuda.current_stream()).cuda_stream
    status = N.lib().rbg_trace(scene.handle, C.byref(rs), C.byref(rr), C.byref(opts), C.c_void_p(st_ptr))
    if check and status not in (N.RBG_OK, N.RBG_ERR_CAP):
        N.check(status, "rbg_trace")
    return res, status


def trace_async(manager, rays, res=None, precision: Optional[int] = None, stream=None, workspace_buf="auto"):
    """rbg_trace_async: the trace of `trace` put on the stream without
    waiting (capturable into a CUDA graph); rbg_trace_status (status())
    reads its status later.  The scene must be on the device already
    (reserve(), or an earlier trace).  Returns the result dict."""
    torch = _torch()
    scene = manager._ensure_scene()
    n = rays["x"].numel()
    if res is None:
        res = alloc_result(n, rays["x"].device)
    opts = manager.trace_options(precision)
    ws = workspace(n, rays["x"].device) if isinstance(workspace_buf, str) else workspace_buf
    if ws is not None:
        opts.workspace = ws.data_ptr()
        opts.workspace_bytes = ws.numel()
    st_ptr = (stream if stream is not None else torch.cuda.current_stream()).cuda_stream
    N.check(N.lib().rbg_trace_async(scene.handle, C.byref(_rays_struct(rays)), C.byref(_result_struct(res)),
                                    C.byref(opts), C.c_void_p(st_ptr)), "rbg_trace_async")
    return res


def status(manager, stream=None) -> int:
    """rbg_trace_status: the status of the scene's last trace on `stream`."""
    torch = _torch()
    st_ptr = (stream if stream is not None else torch.cuda.current_stream()).cuda_stream
    return int(N.lib().rbg_trace_status(manager._ensure_scene().handle, C.c_void_p(st_ptr)))


def autotune(manager, rays, res=None, stream=None) -> int:
    """Pick the mixed tracer's block size and compaction threshold for this
    scene from a timed trace of `rays` per candidate (rbg_scene_autotune);
    later traces of the scene use them.  Returns the chosen threshold
    (tuning() gives both)."""
    torch = _torch()
    scene = manager._ensure_scene()
    if res is None:
        res = alloc_result(rays["x"].numel(), rays["x"].device)
    opts = manager.trace_options(N.PREC_MIXED)
    ws = workspace(rays["x"].numel(), rays["x"].device)
    if ws is not None:
        opts.workspace = ws.data_ptr()
        opts.workspace_bytes = ws.numel()
    st_ptr = (stream if stream is not None else torch.cuda.current_stream()).cuda_stream
    chosen = C.c_int32(0)
    status = N.lib().rbg_scene_autotune(scene.handle, C.byref(_rays_struct(rays)), C.byref(_result_struct(res)),
                                        C.byref(opts), C.c_void_p(st_ptr), C.byref(chosen))
    if status not in (N.RBG_OK, N.RBG_ERR_CAP, N.RBG_ERR_NAN):
        N.check(status, "rbg_scene_autotune")
    return int(chosen.value)


def tuning(manager):
    """(block size, compaction threshold) of the mixed tracer for the scene
    (rbg_scene_tuning: the autotuner's choice, else the defaults)."""
    scene = manager._ensure_scene()
    b, c = C.c_int32(0), C.c_int32(0)
    N.check(N.lib().rbg_scene_tuning(scene.handle, C.byref(b), C.byref(c)), "rbg_scene_tuning")
    return int(b.value), int(c.value)


def focal_moments(res, group=None, n_groups: int = 1, stream=None):
    """(count, sum x, sum y, sum x^2, sum y^2, sum t) of focused rays per group."""
    torch = _torch()
    n = res["x"].numel()
    sums = torch.zeros((n_groups, 6), dtype=torch.float64, device=res["x"].device)
    st = (stream if stream is not None else torch.cuda.current_stream()).cuda_stream
    N.check(N.lib().rbg_focal_moments(n, _ptr(res["status"]), _ptr(res["x"]), _ptr(res["y"]), _ptr(res["t"]),
                                      _ptr(group), n_groups, _ptr(sums), C.c_void_p(st)), "rbg_focal_moments")
    return sums


def focal_histogram(res, nx, xlo, xhi, ny, ylo, yhi, mask=None, stream=None):
    torch = _torch()
    status = res["status"]
    if mask is not None:
        status = torch.where(mask, status, torch.zeros_like(status))
    counts = torch.zeros((nx, ny), dtype=torch.float64, device=res["x"].device)
    st = (stream if stream is not None else torch.cuda.current_stream()).cuda_stream
    N.check(N.lib().rbg_focal_histogram(res["x"].numel(), _ptr(status), _ptr(res["x"]), _ptr(res["y"]), nx, xlo,
                                        xhi, ny, ylo, yhi, _ptr(counts), C.c_void_p(st)), "rbg_focal_histogram")
    return counts


def reserve(manager, max_rays: int, history: int = 0):
    """rbg_scene_reserve: make every device allocation tracing batches of up
    to `max_rays` rays needs, so that later traces allocate nothing."""
    _torch()
    scene = manager._ensure_scene()
    N.check(N.lib().rbg_scene_reserve(scene.handle, int(max_rays), int(history)), "rbg_scene_reserve")


def containment_radius_async(counts, xlo, xhi, ylo, yhi, fraction=0.8, out=None, stream=None):
    """AGeoUtil::ContainmentRadius of a device histogram into a device
    tensor (r, x, y, status), stream-ordered (one launch, no host sync)."""
    torch = _torch()
    counts = counts.contiguous()
    nx, ny = counts.shape
    if out is None:
        out = torch.empty(4, dtype=torch.float64, device=counts.device)
    st = (stream if stream is not None else torch.cuda.current_stream()).cuda_stream
    N.check(N.lib().rbg_containment_radius_async(_ptr(counts), nx, xlo, xhi, ny, ylo, yhi, fraction, _ptr(out),
                                                 C.c_void_p(st)), "rbg_containment_radius_async")
    return out


def containment_radius(counts, xlo, xhi, ylo, yhi, fraction=0.8, stream=None):
    """AGeoUtil::ContainmentRadius of a device histogram -> (r, x, y)."""
    torch = _torch()
    counts = counts.contiguous()
    nx, ny = counts.shape
    r, x, y = C.c_double(), C.c_double(), C.c_double()
    st = (stream if stream is not None else torch.cuda.current_stream()).cuda_stream
    N.check(N.lib().rbg_containment_radius(_ptr(counts), nx, xlo, xhi, ny, ylo, yhi, fraction, C.byref(r),
                                           C.byref(x), C.byref(y), C.c_void_p(st)), "rbg_containment_radius")
    return r.value, x.value, y.value


def shoot(kind: int, params, n: int, lam: float, rot=None, tr=None, v=None, seed=None, first_id: int = 0,
          device="cuda:0", stream=None):
    """An ARayShooter source (rbg_shoot's kinds and parameters) generated on
    the GPU by rbg_shoot_device: a dict of device tensors x, y, z, t, dx,
    dy, dz, lam holding the same rays the host generator draws."""
    torch = _torch()
    from .manager import ARayShooter

    cap = int(n)
    if kind == N.RBG_SHOOT_CIRCLE:
        cap = 1 + int(params[2]) * int(params[1]) * (int(params[1]) + 1) // 2
    elif kind == N.RBG_SHOOT_RECTANGLE:
        cap = int(params[2]) * int(params[3])
    out = {f: torch.empty(cap, dtype=torch.float64, device=device) for f in RAY_FIELDS}
    rays = _rays_struct(out)
    dp = C.POINTER(C.c_double)
    p = (C.c_double * max(1, len(params)))(*params)
    r9 = (C.c_double * 9)(*rot.R.reshape(-1)) if rot is not None else None
    t3 = (C.c_double * 3)(*tr.t) if tr is not None else None
    d3 = (C.c_double * 3)(*[float(a) for a in v]) if v is not None else None
    s = ARayShooter.seed if seed is None else seed
    st = (stream if stream is not None else torch.cuda.current_stream()).cuda_stream
    N.check(N.lib().rbg_shoot_device(kind, C.cast(p, dp), int(n), C.cast(r9, dp) if r9 else None,
                                     C.cast(t3, dp) if t3 else None, C.cast(d3, dp) if d3 else None, s,
                                     first_id, lam, C.byref(rays), C.c_void_p(st)), "rbg_shoot_device")
    m = rays.n
    return {f: t[:m] for f, t in out.items()}


def set_tuning(manager, block_size: int = 0, compaction: int = 0):
    """rbg_scene_set_tuning: the mixed tracer's block size and compaction
    threshold for the scene, set directly."""
    scene = manager._ensure_scene()
    N.check(N.lib().rbg_scene_set_tuning(scene.handle, int(block_size), int(compaction)), "rbg_scene_set_tuning")


# event kinds of rbg_trace_count_events, in the order of the counts
EVENT_KINDS = ("segment", "ray", "xform_t", "xform_g", "polish", "horner64", "accept", "normal", "normal_exact",
               "contains_exact", "box64", "dist_exact", "wall_exact", "reflect", "newton32", "horner32", "screen32")


def count_events(manager, rays, res=None, stream=None):
    """rbg_trace_count_events: the mixed trace of `rays` through the
    counting build.  Returns (counts per event kind, FP64 flops, FP32
    flops) of the whole trace."""
    torch = _torch()
    L = N.lib()
    scene = manager._ensure_scene()
    n = rays["x"].numel()
    if res is None:
        res = alloc_result(n, rays["x"].device)
    opts = manager.trace_options(N.PREC_MIXED)
    ws = workspace(n, rays["x"].device)
    if ws is not None:
        opts.workspace = ws.data_ptr()
        opts.workspace_bytes = ws.numel()
    k = L.rbg_event_kinds()
    counts = (C.c_uint64 * k)()
    st = (stream if stream is not None else torch.cuda.current_stream()).cuda_stream
    N.check(L.rbg_trace_count_events(scene.handle, C.byref(_rays_struct(rays)), C.byref(_result_struct(res)),
                                     C.byref(opts), C.c_void_p(st), counts, k), "rbg_trace_count_events")
    f64 = f32 = 0.0
    for i in range(k):
        a, b = C.c_double(), C.c_double()
        N.check(L.rbg_event_flops(i, C.byref(a), C.byref(b)), "rbg_event_flops")
        f64 += counts[i] * a.value
        f32 += counts[i] * b.value
    return [int(c) for c in counts], f64, f32
