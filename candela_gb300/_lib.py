"""ctypes binding of librq.so (include/rq.h).

The library is the product: there is no Python or CPU implementation of any query behind this
module.  Importing succeeds without a GPU (the tests check the exports on CPU), but every call
that needs the device fails with RQ_ECUDA when there is none, and a missing librq.so raises
ImportError instead of falling back to anything.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "librq.so"

RQ_OK, RQ_EINVAL, RQ_ENOMEM, RQ_ECUDA, RQ_EBUDGET, RQ_ENOTSUP, RQ_ESTATE = range(7)
LAYOUT_DEFAULT, LAYOUT_STACK, LAYOUT_STACKLESS, LAYOUT_BVH8Q = range(4)
MODE_STRICT, MODE_FAST = 0, 1
TIE_LOWER_INDEX, TIE_FIRST_FOUND = 0, 1
FLAG_REF_COMPAT, FLAG_IGNORE_TRANSPARENT, FLAG_HOST_BUFFERS, FLAG_NO_PERSISTENT = 1, 2, 4, 8
FLAG_COUNT = 16
FLAG_ENTITY_LOOP = 32
PIXELS_RGBA32F, PIXELS_RGBA16F = 0, 1
ABI_VERSION = 3

VERTEX_DTYPE = np.dtype([("pos", "<f4", (4,)), ("packed", "<u4", (4,))])
TRI_DTYPE = np.dtype(("<i4", (4,)))
STACK_NODE_DTYPE = np.dtype(("<f4", (16,)))
STACKLESS_NODE_DTYPE = np.dtype(("<f4", (8,)))
ENTITY_DTYPE = np.dtype([("model", "<f4", (16,)), ("inverse", "<f4", (16,)),
                         ("node_offset", "<i4"), ("node_count", "<i4"), ("data", "<i4", (14,))])
RAY_DTYPE = np.dtype([("o", "<f4", (3,)), ("tmin", "<f4"), ("d", "<f4", (3,)), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("w", "<f4"),
                      ("tri", "<i4"), ("mesh", "<i4"), ("entity", "<i4"), ("iters", "<i4")])
assert ENTITY_DTYPE.itemsize == 192 and RAY_DTYPE.itemsize == 32 and HIT_DTYPE.itemsize == 32


class RqOpts(C.Structure):
    _fields_ = [("layout", C.c_int32), ("mode", C.c_int32), ("tie", C.c_int32),
                ("flags", C.c_int32), ("block_size", C.c_int32), ("min_blocks", C.c_int32),
                ("persistent", C.c_int32), ("stack_depth", C.c_int32)]


MAX_VARIANTS = 10
MAX_BATCH_COMBOS = 16


class RqTuneResult(C.Structure):
    _fields_ = [("variant", C.c_int32), ("block_size", C.c_int32), ("min_blocks", C.c_int32),
                ("persistent", C.c_int32), ("n_variants", C.c_int32), ("depth", C.c_int32),
                ("ms", C.c_float * MAX_VARIANTS), ("block", C.c_int32 * MAX_VARIANTS),
                ("min_blocks_of", C.c_int32 * MAX_VARIANTS), ("persistent_of", C.c_int32 * MAX_VARIANTS),
                ("depth_of", C.c_int32 * MAX_VARIANTS)]


class RqBuildOpts(C.Structure):
    _fields_ = [("leaf_size", C.c_int32), ("swap_children", C.c_int32),
                ("swap_seed", C.c_uint32), ("n_threads", C.c_int32)]


class RqBvhInfo(C.Structure):
    _fields_ = [("n_nodes", C.c_int64), ("n_nodes_used", C.c_int64), ("n_tris", C.c_int64),
                ("node_bytes", C.c_int32), ("layout", C.c_int32), ("leaf_count", C.c_int64),
                ("split_fails", C.c_int64), ("build_ms", C.c_double)]


class RqBvh8Info(C.Structure):
    _fields_ = [("nodes", C.c_int64), ("triangles", C.c_int64), ("bytes", C.c_int64),
                ("bvh2_nodes", C.c_int64), ("build_ms", C.c_double)]


class RqDiffParams(C.Structure):
    _fields_ = [("sun_dir", C.c_float * 3), ("sun_color", C.c_float), ("albedo", C.c_float),
                ("w_depth", C.c_float), ("w_radiance", C.c_float), ("shadow_rays", C.c_int32),
                ("shadow_offset", C.c_float), ("recompute", C.c_int32), ("layout", C.c_int32),
                ("reserved", C.c_int32)]


class RqQuery(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("rays", C.c_void_p), ("n", C.c_int64), ("kind", C.c_int32),
                ("reserved", C.c_int32), ("hits", C.c_void_p), ("occluded", C.c_void_p)]


class RqBatchTune(C.Structure):
    _fields_ = [("family", C.c_int32), ("block_size", C.c_int32), ("min_blocks", C.c_int32),
                ("n", C.c_int32), ("depth", C.c_int32), ("ms", C.c_float * MAX_BATCH_COMBOS),
                ("family_of", C.c_int32 * MAX_BATCH_COMBOS), ("block_of", C.c_int32 * MAX_BATCH_COMBOS),
                ("min_blocks_of", C.c_int32 * MAX_BATCH_COMBOS), ("depth_of", C.c_int32 * MAX_BATCH_COMBOS)]


class RqGiParams(C.Structure):
    _fields_ = [("spp", C.c_int32), ("seed", C.c_uint32), ("origin_offset", C.c_float),
                ("ray_tmax", C.c_float), ("normal_mode", C.c_int32), ("query", C.c_int32),
                ("shadow_rays", C.c_int32), ("shadow_offset", C.c_float),
                ("sun_dir", C.c_float * 3), ("sun_color", C.c_float * 3),
                ("sky_color", C.c_float * 3), ("sort_rays", C.c_int32), ("unfused", C.c_int32),
                ("bounces", C.c_int32), ("compact_below", C.c_float), ("pixel_format", C.c_int32)]


class RqGiTune(C.Structure):
    _fields_ = [("compact_below", C.c_float), ("live_fraction", C.c_float), ("ms_compact", C.c_float),
                ("ms_in_place", C.c_float)]


class RqTexture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("srgb", C.c_int32), ("wrap", C.c_int32),
                ("rgba8", C.c_void_p)]


class RqSpecularParams(C.Structure):
    _fields_ = [("seed", C.c_uint32), ("roughness", C.c_float), ("ray_tmax", C.c_float),
                ("normal_mode", C.c_int32), ("shadow_rays", C.c_int32), ("shadow_offset", C.c_float),
                ("sun_dir", C.c_float * 3), ("sun_color", C.c_float * 3), ("sky_color", C.c_float * 3),
                ("ambient", C.c_float * 3)]


class RqProbeParams(C.Structure):
    _fields_ = [("grid", C.c_int32 * 3), ("origin", C.c_float * 3), ("prev_origin", C.c_float * 3),
                ("size", C.c_float * 3), ("seed", C.c_uint32), ("temporal", C.c_int32), ("normal_mode", C.c_int32),
                ("shadow_rays", C.c_int32), ("shadow_offset", C.c_float), ("ray_tmax", C.c_float),
                ("sun_dir", C.c_float * 3), ("sun_color", C.c_float * 3), ("sky_color", C.c_float * 3)]


class RqFrameStats(C.Structure):
    _fields_ = [("primary_rays", C.c_int64), ("primary_hits", C.c_int64),
                ("secondary_rays", C.c_int64), ("secondary_hits", C.c_int64),
                ("shadow_rays", C.c_int64), ("shadow_occluded", C.c_int64),
                ("bounce_rays", C.c_int64), ("bounce_hits", C.c_int64)]


_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int32
_S = C.c_int

# name -> (restype, argtypes).  Every symbol declared in include/rq.h appears here.
SIGNATURES = {
    "rq_abi_version": (C.c_int, []),
    "rq_status_string": (C.c_char_p, [_S]),
    "rq_create": (_S, [C.c_int, C.POINTER(_P)]),
    "rq_destroy": (_S, [_P]),
    "rq_last_error": (C.c_char_p, [_P]),
    "rq_build_bvh": (_S, [_P, _I64, _P, _I64, _P, _I32, _S, C.POINTER(RqBuildOpts), C.POINTER(_P)]),
    "rq_build_bvh_gpu": (_S, [_P, _P, _I64, _P, _I64, _P, _I32, _S, C.POINTER(RqBuildOpts), C.POINTER(_P)]),
    "rq_bvh_info_get": (_S, [_P, C.POINTER(RqBvhInfo)]),
    "rq_bvh_nodes": (_S, [_P, C.POINTER(_P), C.POINTER(_I64)]),
    "rq_bvh_triangles": (_S, [_P, C.POINTER(_P), C.POINTER(_I64)]),
    "rq_bvh_free": (None, [_P]),
    "rq_scene_validate": (_S, [_S, _P, _I64, _P, _I64, _P, _I64, _P, _I32, C.c_char_p, C.c_size_t]),
    "rq_scene_create": (_S, [_P, _S, _P, _I64, _P, _I64, _P, _I64, _P, _I32, C.POINTER(_P)]),
    "rq_scene_set_entities": (_S, [_P, _P, _I32]),
    "rq_scene_bytes": (_S, [_P, C.POINTER(_I64)]),
    "rq_scene_destroy": (_S, [_P]),
    "rq_closest": (_S, [_P, _P, _P, _I64, _P, C.POINTER(RqOpts), _P]),
    "rq_anyhit": (_S, [_P, _P, _P, _I64, _P, C.POINTER(RqOpts), _P]),
    "rq_counters_read": (_S, [_P, C.POINTER(C.c_int64 * 2), C.c_int]),
    "rq_device_status": (_S, [_P, C.POINTER(C.c_uint32), C.c_int]),
    "rq_autotune": (_S, [_P, _P, _P, _I64, _I32, _S, C.POINTER(RqTuneResult)]),
    "rq_scene_build_bvh8": (_S, [_P, C.POINTER(RqBvh8Info)]),
    "rq_build_bvh8": (_S, [_S, _P, _I64, _P, _I64, _P, _I64, _I32, _I32, C.POINTER(_P)]),
    "rq_bvh8_buffers": (_S, [_P, C.POINTER(_P), C.POINTER(_I64), C.POINTER(_P), C.POINTER(_I64)]),
    "rq_bvh8_free": (None, [_P]),
    "rq_scene_set_materials": (_S, [_P, _P, _I32]),
    "rq_gi_raygen": (_S, [_P, _P, _P, _P, _I64, C.POINTER(RqGiParams), _P, _P]),
    "rq_shadow_raygen": (_S, [_P, _P, _P, _P, _I64, C.POINTER(RqGiParams), _P, _P]),
    "rq_shade": (_S, [_P, _P, _P, _P, _I64, _P, C.POINTER(RqGiParams), _P, _P]),
    "rq_gi_frame": (_S, [_P, _P, _P, _I64, C.POINTER(RqGiParams), C.POINTER(RqOpts), _P,
                         C.POINTER(RqFrameStats), _P]),
    "rq_fwd": (_S, [_P, _P, _P, _I64, _P, C.POINTER(RqDiffParams), _P, C.POINTER(C.c_double),
                    C.POINTER(_P), _P]),
    "rq_bwd": (_S, [_P, _P, _P, _P]),
    "rq_tape_free": (_S, [_P]),
    "rq_tape_bytes": (_S, [_P, C.POINTER(_I64)]),
    "rq_scene_update_positions": (_S, [_P, _P, _P]),
    "rq_verify_hits": (_S, [_P, _P, _P, _P, _I64, _P, _P]),
    "rq_batch": (_S, [_P, C.POINTER(RqQuery), _I32, C.POINTER(RqOpts), _P]),
    "rq_batch_plan_create": (_S, [_P, C.POINTER(RqQuery), _I32, C.POINTER(RqOpts), C.POINTER(_P)]),
    "rq_batch_plan_launch": (_S, [_P, _P]),
    "rq_batch_plan_autotune": (_S, [_P, _I32, C.POINTER(RqBatchTune)]),
    "rq_batch_plan_destroy": (_S, [_P]),
    "rq_gi_frame_noalloc": (_S, [_P, _P, _P, _I64, C.POINTER(RqGiParams), C.POINTER(RqOpts), _P,
                                 _P]),
    "rq_collide": (_S, [_P, _P, _P, _I64, _P, C.POINTER(RqOpts), _P]),
    "rq_scene_tlas_info": (_S, [_P, C.POINTER(C.c_int64 * 3)]),
    "rq_scene_set_textures": (_S, [_P, _P, _I32, _P, _I32]),
    "rq_specular_frame": (_S, [_P, _P, _P, _I64, C.POINTER(RqSpecularParams), C.POINTER(RqOpts), _P, _P]),
    "rq_probe_update": (_S, [_P, _P, C.POINTER(RqProbeParams), _P, _P, _P, _P, _P, C.POINTER(RqOpts), _P]),
    "rq_measure_read_gbs": (_S, [_P, _I64, _I32, C.POINTER(C.c_double)]),
    "rq_hit_attribs": (_S, [_P, _P, _P, _I64, _P, C.POINTER(RqOpts), _P]),
    "rq_closest_attribs": (_S, [_P, _P, _P, _I64, _P, _P, C.POINTER(RqOpts), _P]),
    "rq_gi_autotune": (_S, [_P, _P, _P, _I64, C.POINTER(RqGiParams), C.POINTER(RqOpts), _P, C.POINTER(RqGiTune)]),
}

NOALLOC_MAX_RAYS = 65536

_lib = None


def lib() -> C.CDLL:
    """Loads librq.so once.  Raises ImportError when it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run candela_gb300._build.build() "
                              "(the engine has no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class RqError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


def check(status: int, ctx=None) -> None:
    if status != RQ_OK:
        m = lib().rq_last_error(ctx)
        raise RqError(status, (m or b"").decode() or lib().rq_status_string(status).decode())


def ptr(a) -> int:
    """Address of a numpy array's data or of a torch tensor's storage."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"
        return a.ctypes.data
    return a.data_ptr()
