"""ctypes mirror of include/robast_gb.h and loaders for the native libraries.

The product library (``librobast_gb.so``: scene flattener, CUDA kernels and
the C ABI) is built in-tree by :mod:`robast_gb300.build`.  Loading fails
loudly when it is missing: there is no Python or CPU fallback for tracing.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(_HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "librobast_gb.so")

# ---- constants (robast_gb.h) -------------------------------------------
RBG_OK, RBG_ERR_ARG, RBG_ERR_SCENE, RBG_ERR_CUDA, RBG_ERR_NAN = 0, 1, 2, 3, 4
RBG_ERR_CAP, RBG_ERR_UNSUPPORTED, RBG_ERR_NOMEM, RBG_ERR_NODEVICE = 5, 6, 7, 8
RBG_ERR_TOO_LARGE = 9

RBG_RUN, RBG_STOP, RBG_EXIT, RBG_FOCUS, RBG_SUSPEND, RBG_ABSORB = range(6)

KIND_LENS, KIND_OBS, KIND_MIRROR, KIND_FOCUS, KIND_OPT, KIND_OTHER = range(6)

SHAPE_BOX, SHAPE_TUBE, SHAPE_SPHERE, SHAPE_PARABOLOID = 1, 2, 3, 4
SHAPE_PGON, SHAPE_PCON, SHAPE_ASPHERIC_DISK, SHAPE_WINSTON_POLY = 5, 6, 7, 8
SHAPE_COMPOSITE = 9
SHAPE_WINSTON_2D = 10
OP_UNION, OP_INTERSECTION, OP_SUBTRACTION = 0, 1, 2

TABLE_1D, TABLE_2D = 1, 2
INDEX_TABLE, INDEX_SELLMEIER, INDEX_CAUCHY, INDEX_SCHOTT, INDEX_MIXED = 1, 2, 3, 4, 5

PREC_FP64, PREC_MIXED = 0, 1
ORDER_SPATIAL, ORDER_INPUT = 0, 1


class ShapeDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("param_offset", C.c_int32), ("n_params", C.c_int32),
                ("op", C.c_int32), ("left", C.c_int32), ("right", C.c_int32),
                ("left_matrix", C.c_int32), ("right_matrix", C.c_int32)]


class TableDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32),
                ("param_offset", C.c_int32)]


class IndexDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("n_table", C.c_int32), ("k_table", C.c_int32),
                ("mix_a", C.c_int32), ("mix_b", C.c_int32), ("coef", C.c_double * 6)]


class LayerDesc(C.Structure):
    _fields_ = [("index", C.c_int32), ("coherent", C.c_int32), ("thickness", C.c_double)]


class MultilayerDesc(C.Structure):
    _fields_ = [("layer_offset", C.c_int32), ("n_layers", C.c_int32), ("precalc", C.c_int32),
                ("lam_nbins", C.c_int32), ("th_nbins", C.c_int32), ("reserved", C.c_int32),
                ("lam_min", C.c_double), ("lam_max", C.c_double), ("th_min", C.c_double), ("th_max", C.c_double)]


class BorderDesc(C.Structure):
    _fields_ = [("component1", C.c_int32), ("component2", C.c_int32), ("sigma", C.c_double),
                ("multilayer", C.c_int32), ("lambertian", C.c_int32)]


class VolumeDesc(C.Structure):
    _fields_ = [("shape", C.c_int32), ("kind", C.c_int32), ("reflectance", C.c_double),
                ("refl_table", C.c_int32), ("index", C.c_int32),
                ("qe_lambda_table", C.c_int32), ("qe_angle_table", C.c_int32)]


class PlacementDesc(C.Structure):
    _fields_ = [("mother", C.c_int32), ("daughter", C.c_int32), ("matrix", C.c_int32),
                ("copy_no", C.c_int32), ("overlap", C.c_int32)]


class SceneDesc(C.Structure):
    _fields_ = [
        ("n_shapes", C.c_int32), ("shapes", C.POINTER(ShapeDesc)),
        ("n_matrices", C.c_int32), ("matrices", C.POINTER(C.c_double)),
        ("n_volumes", C.c_int32), ("volumes", C.POINTER(VolumeDesc)),
        ("n_placements", C.c_int32), ("placements", C.POINTER(PlacementDesc)),
        ("top_volume", C.c_int32),
        ("n_tables", C.c_int32), ("tables", C.POINTER(TableDesc)),
        ("n_indices", C.c_int32), ("indices", C.POINTER(IndexDesc)),
        ("n_layers", C.c_int32), ("layers", C.POINTER(LayerDesc)),
        ("n_multilayers", C.c_int32), ("multilayers", C.POINTER(MultilayerDesc)),
        ("n_borders", C.c_int32), ("borders", C.POINTER(BorderDesc)),
        ("n_params", C.c_int64), ("params", C.POINTER(C.c_double)),
    ]


class Node(C.Structure):
    _fields_ = [("parent", C.c_int32), ("volume", C.c_int32), ("shape", C.c_int32),
                ("kind", C.c_int32), ("child_begin", C.c_int32), ("child_count", C.c_int32),
                ("bvh_root", C.c_int32), ("depth", C.c_int32), ("m", C.c_double * 12),
                ("lo", C.c_double * 3), ("hi", C.c_double * 3)]


class BvhNode(C.Structure):
    _fields_ = [("lo", C.c_float * 3), ("hi", C.c_float * 3), ("left", C.c_int32),
                ("right", C.c_int32), ("item_begin", C.c_int32), ("pad", C.c_int32)]


class FlatScene(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_int32), ("nodes", C.POINTER(Node)),
        ("n_children", C.c_int32), ("children", C.POINTER(C.c_int32)),
        ("n_bvh", C.c_int32), ("bvh", C.POINTER(BvhNode)),
        ("n_bvh_items", C.c_int32), ("bvh_items", C.POINTER(C.c_int32)),
        ("n_shapes", C.c_int32), ("shapes", C.POINTER(ShapeDesc)),
        ("n_volumes", C.c_int32), ("volumes", C.POINTER(VolumeDesc)),
        ("n_tables", C.c_int32), ("tables", C.POINTER(TableDesc)),
        ("n_indices", C.c_int32), ("indices", C.POINTER(IndexDesc)),
        ("n_layers", C.c_int32), ("layers", C.POINTER(LayerDesc)),
        ("n_multilayers", C.c_int32), ("multilayers", C.POINTER(MultilayerDesc)),
        ("n_borders", C.c_int32), ("borders", C.POINTER(BorderDesc)),
        ("n_params", C.c_int64), ("params", C.POINTER(C.c_double)),
        ("top_node", C.c_int32),
    ]


_dp = C.POINTER(C.c_double)


class Rays(C.Structure):
    _fields_ = [("n", C.c_int64), ("x", _dp), ("y", _dp), ("z", _dp), ("t", _dp),
                ("dx", _dp), ("dy", _dp), ("dz", _dp), ("lambda_", _dp)]


class Result(C.Structure):
    _fields_ = [("status", C.POINTER(C.c_uint8)), ("npoints", C.POINTER(C.c_int32)),
                ("last_node", C.POINTER(C.c_int32)), ("x", _dp), ("y", _dp), ("z", _dp),
                ("t", _dp), ("dx", _dp), ("dy", _dp), ("dz", _dp), ("hist_cap", C.c_int32),
                ("hist_xyzt", _dp), ("hist_node", C.POINTER(C.c_int32))]


class Bunches(C.Structure):
    _fields_ = [("n", C.c_int64), ("tel", C.POINTER(C.c_int32)), ("array", C.POINTER(C.c_int32))] + \
        [(f, C.POINTER(C.c_float)) for f in ("x", "y", "zem", "time", "cx", "cy", "cz", "lambda_", "photons")]


class TraceOpts(C.Structure):
    _fields_ = [("limit", C.c_int32), ("disable_fresnel", C.c_int32), ("seed", C.c_uint64),
                ("ray_id_offset", C.c_uint64), ("precision", C.c_int32),
                ("block_size", C.c_int32), ("compaction", C.c_int32), ("ray_order", C.c_int32),
                ("workspace", C.c_void_p), ("workspace_bytes", C.c_uint64)]


class NativeError(RuntimeError):
    """Non-zero status from the C ABI."""

    def __init__(self, status: int, what: str, message: str):
        super().__init__(f"{what}: {message} (status {status})")
        self.status = status


_lib = None


def lib():
    """The product library.  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -c \"import robast_gb300.build as b; "
                "b.build_library()\"` (there is no fallback tracer)")
        L = C.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def _declare(L):
    vp = C.c_void_p
    L.rbg_abi_version.restype = C.c_int
    L.rbg_status_string.restype = C.c_char_p
    L.rbg_status_string.argtypes = [C.c_int]
    L.rbg_trace_opts_default.argtypes = [C.POINTER(TraceOpts)]
    L.rbg_scene_create.argtypes = [C.POINTER(SceneDesc), C.POINTER(vp)]
    L.rbg_scene_destroy.argtypes = [vp]
    L.rbg_scene_destroy.restype = None
    L.rbg_scene_flat.argtypes = [vp, C.POINTER(FlatScene)]
    L.rbg_scene_upload.argtypes = [vp]
    L.rbg_scene_reserve.argtypes = [vp, C.c_int64, C.c_int32]
    L.rbg_trace_workspace_bytes.argtypes = [C.c_int64]
    L.rbg_measure_fma_peak.argtypes = [C.c_int32, _dp, vp]
    L.rbg_event_flops.argtypes = [C.c_int32, _dp, _dp]
    L.rbg_trace_count_events.argtypes = [vp, C.POINTER(Rays), C.POINTER(Result), C.POINTER(TraceOpts), vp,
                                         C.POINTER(C.c_uint64), C.c_int32]
    L.rbg_trace_workspace_bytes.restype = C.c_size_t
    L.rbg_trace.argtypes = [vp, C.POINTER(Rays), C.POINTER(Result), C.POINTER(TraceOpts), vp]
    L.rbg_trace_async.argtypes = [vp, C.POINTER(Rays), C.POINTER(Result), C.POINTER(TraceOpts), vp]
    L.rbg_trace_status.argtypes = [vp, vp]
    L.rbg_trace_host.argtypes = [vp, C.POINTER(Rays), C.POINTER(Result), C.POINTER(TraceOpts)]
    L.rbg_scene_autotune.argtypes = [vp, C.POINTER(Rays), C.POINTER(Result), C.POINTER(TraceOpts), vp,
                                     C.POINTER(C.c_int32)]
    L.rbg_scene_tuning.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    L.rbg_scene_set_tuning.argtypes = [vp, C.c_int32, C.c_int32]
    L.rbg_last_launch_count.argtypes = [vp]
    L.rbg_scene_set_timing.argtypes = [vp, C.c_int32]
    L.rbg_last_kernel_ms.argtypes = [vp]
    L.rbg_last_kernel_ms.restype = C.c_double
    L.rbg_multilayer_rt.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int64, vp, vp, vp, vp, vp, vp]
    L.rbg_focal_moments.argtypes = [C.c_int64, vp, vp, vp, vp, vp, C.c_int32, vp, vp]
    L.rbg_focal_histogram.argtypes = [C.c_int64, vp, vp, vp, C.c_int32, C.c_double, C.c_double,
                                      C.c_int32, C.c_double, C.c_double, vp, vp]
    L.rbg_containment_radius.argtypes = [vp, C.c_int32, C.c_double, C.c_double, C.c_int32,
                                         C.c_double, C.c_double, C.c_double, _dp, _dp, _dp, vp]
    L.rbg_containment_radius_async.argtypes = [vp, C.c_int32, C.c_double, C.c_double, C.c_int32,
                                               C.c_double, C.c_double, C.c_double, vp, vp]
    L.rbg_shoot.argtypes = [C.c_int32, _dp, C.c_int64, _dp, _dp, _dp, C.c_uint64, C.c_uint64,
                            C.c_double, C.POINTER(Rays)]
    L.rbg_shoot_device.argtypes = [C.c_int32, _dp, C.c_int64, _dp, _dp, _dp, C.c_uint64, C.c_uint64,
                                   C.c_double, C.POINTER(Rays), vp]
    fp = C.POINTER(C.c_float)
    ip = C.POINTER(C.c_int32)
    L.rbg_corsika_open.argtypes = [C.c_char_p, C.c_int64, C.POINTER(vp)]
    L.rbg_corsika_close.argtypes = [vp]
    L.rbg_corsika_close.restype = None
    L.rbg_corsika_run_header.argtypes = [vp, fp]
    L.rbg_corsika_event_header.argtypes = [vp, fp]
    L.rbg_corsika_input_lines.argtypes = [vp, C.c_char_p, C.c_int64, ip]
    L.rbg_corsika_telescopes.argtypes = [vp, C.c_int32, ip, _dp, _dp, _dp, _dp]
    L.rbg_corsika_read_event.argtypes = [vp, C.c_int32, ip]
    L.rbg_corsika_offsets.argtypes = [vp, C.c_int32, ip, _dp, _dp, _dp]
    L.rbg_corsika_bunch_count.argtypes = [vp, C.c_int32, C.c_int32]
    L.rbg_corsika_bunch_count.restype = C.c_int64
    L.rbg_corsika_get_bunches.argtypes = [vp, C.c_int32, C.c_int32, C.POINTER(Bunches)]
    L.rbg_bunches_workspace_bytes.argtypes = [C.c_int64]
    L.rbg_bunches_workspace_bytes.restype = C.c_size_t
    L.rbg_bunches_to_rays.argtypes = [C.POINTER(Bunches), C.c_double, C.c_double, C.c_double, C.c_double,
                                      C.c_double, C.c_uint64, vp, C.POINTER(Rays), C.c_int64,
                                      C.POINTER(C.c_int64), vp]


def check(status: int, what: str):
    if status != RBG_OK:
        msg = lib().rbg_status_string(status).decode()
        raise NativeError(status, what, msg)


def status_string(status: int) -> str:
    return lib().rbg_status_string(status).decode()

RBG_SHOOT_CIRCLE, RBG_SHOOT_RANDOM_CIRCLE, RBG_SHOOT_RANDOM_CONE = 1, 2, 3
RBG_SHOOT_RANDOM_RECTANGLE, RBG_SHOOT_RANDOM_SPHERE = 4, 5
RBG_SHOOT_RANDOM_SPHERICAL_CONE, RBG_SHOOT_RECTANGLE = 6, 7
