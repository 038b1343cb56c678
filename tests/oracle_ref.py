"""Test-side access to the CPU FP64 oracle (oracle/liboracle.so).

The oracle is test infrastructure: only tests, __graft_entry__.smoke() and
bench.py's CPU baseline call it, always as the checker of the GPU path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from robast_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "liboracle.so")

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            from robast_gb300 import build
            build.build_oracle()
        L = C.CDLL(ORACLE_LIB)
        fs = C.POINTER(N.FlatScene)
        dp = C.POINTER(C.c_double)
        L.orc_trace.argtypes = [fs, C.POINTER(N.Rays), C.POINTER(N.Result), C.POINTER(N.TraceOpts), C.c_int]
        L.orc_coherent_tmm.argtypes = [fs, C.c_int, C.c_int, C.c_double, C.c_double, dp, dp]
        L.orc_coherent_tmm_mixed.argtypes = [fs, C.c_int, C.c_double, C.c_double, dp, dp]
        for f in ("orc_coherent_tmm_c", "orc_incoherent_tmm"):
            getattr(L, f).argtypes = [fs, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, dp, dp]
        L.orc_refractive_index.argtypes = [fs, C.c_int, C.c_double]
        L.orc_refractive_index.restype = C.c_double
        L.orc_extinction.argtypes = [fs, C.c_int, C.c_double]
        L.orc_extinction.restype = C.c_double
        L.orc_mirror_reflectance.argtypes = [fs, C.c_int, C.c_double, C.c_double]
        L.orc_mirror_reflectance.restype = C.c_double
        L.orc_table_eval.argtypes = [fs, C.c_int, C.c_double, C.c_double]
        L.orc_table_eval.restype = C.c_double
        L.orc_philox.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_containment_radius.argtypes = [dp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double,
                                             C.c_double, C.c_double, dp, dp, dp]
        for f in ("orc_shape_dist_out", "orc_shape_dist_in"):
            getattr(L, f).argtypes = [fs, C.c_int, dp, dp]
            getattr(L, f).restype = C.c_double
        L.orc_shape_contains.argtypes = [fs, C.c_int, dp]
        L.orc_bunches_to_rays.argtypes = [C.POINTER(N.Bunches), C.c_double, C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_uint64] + [dp] * 8 + [C.c_int64]
        L.orc_bunches_to_rays.restype = C.c_int64
        _lib = L
    return _lib


def trace(manager, rays, threads: int = 1, history: int = 0, flat: str = "independent"):
    """Trace a copy of `rays` (ARayArray) with the oracle using the manager's
    scene and options.  The oracle reads the scene as flattened
    independently of the product (flat_ref.py) unless flat == "product".
    Returns (status, dict of result arrays)."""
    import flat_ref
    from robast_gb300.manager import make_result

    scene = manager._ensure_scene()
    fs = flat_ref.independent_flat(scene).flat if flat == "independent" else scene.flat
    res, keep = make_result(len(rays), history)
    opts = manager.trace_options()
    rs = rays.rays_struct()
    st = lib().orc_trace(C.byref(fs), C.byref(rs), C.byref(res), C.byref(opts), threads)
    return st, keep


def tmm(manager_or_scene, ml: int, pol, th0: float, lam: float):
    scene = manager_or_scene._ensure_scene() if hasattr(manager_or_scene, "_ensure_scene") else manager_or_scene
    R, T = C.c_double(), C.c_double()
    if pol == "mixed":
        st = lib().orc_coherent_tmm_mixed(C.byref(scene.flat), ml, th0, lam, C.byref(R), C.byref(T))
    else:
        st = lib().orc_coherent_tmm(C.byref(scene.flat), ml, pol, th0, lam, C.byref(R), C.byref(T))
    assert st == 0
    return R.value, T.value


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox(c, k, o)
    return list(o)


def containment_radius(counts: np.ndarray, xlo, xhi, ylo, yhi, fraction):
    counts = np.ascontiguousarray(counts, dtype=np.float64)
    nx, ny = counts.shape
    r, x, y = C.c_double(), C.c_double(), C.c_double()
    lib().orc_containment_radius(counts.ctypes.data_as(C.POINTER(C.c_double)), nx, xlo, xhi, ny, ylo, yhi,
                                 fraction, C.byref(r), C.byref(x), C.byref(y))
    return r.value, x.value, y.value


def bunches_to_rays(b, z, tel_z, n_index, lam_min, lam_max, seed):
    """ACorsikaIACTFile::GetRayArray restated (oracle) on host bunch arrays
    (dict of float32 arrays as ACorsikaIACTFile.GetBunches returns)."""
    fields = ("x", "y", "zem", "time", "cx", "cy", "cz", "lambda", "photons")
    nb = len(b["x"])
    bs = N.Bunches()
    bs.n = nb
    fp = C.POINTER(C.c_float)
    arrs = {f: np.ascontiguousarray(b[f], dtype=np.float32) for f in fields}
    for f in fields:
        setattr(bs, "lambda_" if f == "lambda" else f, arrs[f].ctypes.data_as(fp))
    cap = int(np.sum(np.ceil(np.maximum(arrs["photons"], 0)))) + 1
    out = {f: np.zeros(cap) for f in ("x", "y", "z", "t", "dx", "dy", "dz", "lam")}
    dp = C.POINTER(C.c_double)
    n = lib().orc_bunches_to_rays(C.byref(bs), z, tel_z, n_index, lam_min, lam_max, seed,
                                  *(out[f].ctypes.data_as(dp) for f in ("x", "y", "z", "t", "dx", "dy", "dz", "lam")),
                                  cap)
    return {k: v[:n] for k, v in out.items()}


def tmm_c(manager_or_scene, ml: int, pol: int, th: complex, lam: float, incoherent=False):
    """Oracle CoherentTMM / IncoherentTMM for a complex incidence angle."""
    scene = manager_or_scene._ensure_scene() if hasattr(manager_or_scene, "_ensure_scene") else manager_or_scene
    R, T = C.c_double(), C.c_double()
    f = lib().orc_incoherent_tmm if incoherent else lib().orc_coherent_tmm_c
    st = f(C.byref(scene.flat), ml, pol, complex(th).real, complex(th).imag, lam, C.byref(R), C.byref(T))
    assert st == 0
    return R.value, T.value
