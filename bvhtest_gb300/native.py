"""ctypes binding of libbvhgb.so (the C ABI declared in include/bvhgb.h).

The library is the only compute path: if it is missing or fails to load, every call raises. There
is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libbvhgb.so"

NODE_DTYPE = np.dtype([
    ("mn", "<f4", (3,)), ("mx", "<f4", (3,)), ("parent", "<u4"), ("left", "<u4"), ("right", "<u4"),
    ("isLeafFlag", "<u2"), ("isLeft", "<u2"), ("level", "<u2"), ("pad", "<u2"), ("surfaceArea", "<f4"),
])
PIXEL_DTYPE = np.dtype([("hit", "u1"), ("diffuse", "u1"), ("intCount", "<u2")])
HIT_DTYPE = np.dtype([("prim", "<u4"), ("t", "<f4")])

STATUS = {0: "OK", 1: "WARNING", 2: "IO_ERROR", 3: "PARSE_ERROR", 4: "BVH_ERROR", 5: "GL_ERROR", 6: "CUDA_ERROR",
          7: "GENERIC_ERROR", 8: "INVALID_ARGUMENT", 9: "DEVICE_TIMEOUT", 10: "OUT_OF_MEMORY", 11: "TOO_LARGE"}


class BvhgbError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)}" + (f" ({detail})" if detail else ""))


class Aabb(C.Structure):
    _fields_ = [("mn", C.c_float * 3), ("mx", C.c_float * 3)]


class LbvhConfig(C.Structure):
    _fields_ = [("mortonBits", C.c_uint32), ("topology", C.c_uint32)]


class Bn13Config(C.Structure):
    _fields_ = [("numChunks", C.c_uint32), ("blockSize", C.c_uint32), ("batchPercent", C.c_float),
                ("offsetAccess", C.c_uint32), ("heapCapacity", C.c_uint32), ("profileKernels", C.c_uint32),
                ("searchMode", C.c_uint32), ("chunkSize", C.c_uint32)]


class Bn13Stats(C.Structure):
    _fields_ = [("items", C.c_uint64), ("applied", C.c_uint64), ("skippedConflict", C.c_uint64),
                ("skippedInvalid", C.c_uint64), ("heapOverflow", C.c_uint64), ("nodesVisited", C.c_uint64)]


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("lookAt", C.c_float * 3), ("up", C.c_float * 3), ("fov", C.c_float),
                ("width", C.c_uint32), ("height", C.c_uint32)]


class TraceConfig(C.Structure):
    _fields_ = [("light", C.c_float * 3), ("faceCulling", C.c_uint32), ("tmin", C.c_float), ("tmax", C.c_float),
                ("rayBundles", C.c_uint32)]


class BatchConfig(C.Structure):
    _fields_ = [("mortonBits", C.c_uint32), ("topology", C.c_uint32), ("numChunks", C.c_uint32),
                ("batchPercent", C.c_float), ("sortTileKeys", C.c_uint32), ("refitBlock", C.c_uint32),
                ("traceBlock", C.c_uint32)]


class BatchTuneReport(C.Structure):
    _fields_ = [("sortTileKeys", C.c_uint32 * 3), ("sortTileMs", C.c_float * 3), ("refitBlock", C.c_uint32 * 3),
                ("refitBlockMs", C.c_float * 3), ("traceBlock", C.c_uint32 * 3), ("traceBlockMs", C.c_float * 3),
                ("chosen", BatchConfig)]


class MeshRaw(C.Structure):
    _fields_ = [("vert", C.c_void_p), ("norm", C.c_void_p), ("faces", C.c_void_p), ("numVert", C.c_uint32),
                ("numNorm", C.c_uint32), ("numFaces", C.c_uint32)]


class BvhPointer(C.Structure):
    _fields_ = [("bvh", C.c_void_p), ("nodes", C.c_void_p), ("numNodes", C.c_uint32)]


VP, U32, U64, I32, F32, SZ = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_float, C.c_size_t
PROTOS = {
    "bvhgb_version": (C.c_char_p, []),
    "bvhgb_status_string": (C.c_char_p, [I32]),
    "bvhgb_last_error": (C.c_char_p, []),
    "bvhgb_launch_count": (U64, []),
    "bvhgb_lbvh_create": (I32, [U32, C.POINTER(LbvhConfig), C.POINTER(VP)]),
    "bvhgb_lbvh_destroy": (I32, [VP]),
    "bvhgb_lbvh_build": (I32, [VP, VP, VP, U32, VP, VP]),
    "bvhgb_lbvh_init_tri_data": (I32, [VP, VP, VP, U32, VP]),
    "bvhgb_lbvh_calc_morton": (I32, [VP, VP, VP, U32, VP]),
    "bvhgb_lbvh_sort": (I32, [VP, U32, VP]),
    "bvhgb_lbvh_build_tree": (I32, [VP, VP, VP, U32, VP, VP]),
    "bvhgb_lbvh_read_scene_box": (I32, [VP, C.POINTER(Aabb), VP]),
    "bvhgb_lbvh_set_scene_box": (I32, [VP, C.POINTER(Aabb), VP]),
    "bvhgb_lbvh_read_keys": (I32, [VP, I32, VP, VP, U32, VP]),
    "bvhgb_lbvh_read_errors": (I32, [VP, C.POINTER(U32), VP]),
    "bvhgb_radix_sort_pairs": (I32, [VP, C.POINTER(SZ), VP, VP, VP, VP, U32, U32, U32, U32, VP]),
    "bvhgb_select_smallest_pairs": (I32, [VP, C.POINTER(SZ), VP, VP, VP, U32, U32, VP]),
    "bvhgb_sort_set_default_tile": (I32, [U32, C.POINTER(U32)]),
    "bvhgb_sort_set_spin_limit": (I32, [U32, C.POINTER(U32)]),
    "bvhgb_debug_fail_allocations": (I32, [C.c_int64, C.POINTER(C.c_int64)]),
    "bvhgb_calc_sah": (I32, [VP, U32, U32, C.POINTER(C.c_double), VP]),
    "bvhgb_bn13_create": (I32, [VP, U32, U32, C.POINTER(Bn13Config), C.POINTER(VP), VP]),
    "bvhgb_bn13_destroy": (I32, [VP]),
    "bvhgb_bn13_step": (I32, [VP, VP, VP]),
    "bvhgb_bn13_run": (I32, [VP, VP, U32, VP]),
    "bvhgb_bn13_select_nodes": (I32, [VP, VP, VP]),
    "bvhgb_bn13_chunk": (I32, [VP, VP, U32, VP]),
    "bvhgb_bn13_get_stats": (I32, [VP, C.POINTER(Bn13Stats), VP]),
    "bvhgb_bn13_refit": (I32, [VP, VP, VP]),
    "bvhgb_bn13_batch_size": (U32, [VP]),
    "bvhgb_bn13_launches_per_iteration": (U32, [VP]),
    "bvhgb_bn13_search_time": (I32, [VP, C.POINTER(F32), C.POINTER(U32)]),
    "bvhgb_bn13_gains": (I32, [VP, VP, VP, U32, VP, VP, VP]),
    "bvhgb_bn13_read_inner": (I32, [VP, VP, U32, C.POINTER(U32), VP]),
    "bvhgb_bn13_set_scorer": (I32, [VP, VP, U32]),
    "bvhgb_bn13_iteration": (U64, [VP]),
    "bvhgb_bn13_set_iteration": (I32, [VP, U64]),
    "bvhgb_bn13_set_tail_packing": (I32, [VP, U32]),
    "bvhgb_bn13_read_selection": (I32, [VP, VP, U32, VP]),
    "bvhgb_bn13_set_selection": (I32, [VP, VP, U32, VP]),
    "bvhgb_batch_create": (I32, [U32, VP, C.POINTER(BatchConfig), C.POINTER(VP)]),
    "bvhgb_batch_destroy": (I32, [VP]),
    "bvhgb_batch_offsets": (I32, [VP, VP, VP]),
    "bvhgb_batch_get_config": (I32, [VP, C.POINTER(BatchConfig)]),
    "bvhgb_batch_set_config": (I32, [VP, C.POINTER(BatchConfig)]),
    "bvhgb_batch_build": (I32, [VP, VP, VP, VP, VP]),
    "bvhgb_batch_optimize": (I32, [VP, VP, U32, VP]),
    "bvhgb_batch_trace_random": (I32, [VP, VP, VP, VP, U32, U64, VP, VP, VP, VP]),
    "bvhgb_batch_run": (I32, [VP, VP, VP, VP, U32, U32, U64, VP, VP]),
    "bvhgb_batch_get_stats": (I32, [VP, C.POINTER(Bn13Stats), C.POINTER(U32), VP]),
    "bvhgb_batch_autotune": (I32, [VP, VP, VP, VP, U32, U64, VP, C.POINTER(BatchTuneReport), VP]),
    "bvhgb_mlp_create": (I32, [U64, C.POINTER(VP)]),
    "bvhgb_mlp_destroy": (I32, [VP]),
    "bvhgb_mlp_set_params": (I32, [VP, VP]),
    "bvhgb_mlp_get_params": (I32, [VP, VP]),
    "bvhgb_mlp_forward": (I32, [VP, VP, U32, VP, VP]),
    "bvhgb_mlp_read_errors": (I32, [VP, C.POINTER(U32), I32]),
    "bvhgb_mlp_gradient": (I32, [VP, VP, VP, U32, VP, VP, VP]),
    "bvhgb_mlp_train": (I32, [VP, VP, VP, U32, U32, U32, F32, F32, U64, VP, VP]),
    "bvhgb_lr_features_create": (I32, [U32, C.POINTER(VP)]),
    "bvhgb_lr_features_destroy": (I32, [VP]),
    "bvhgb_lr_features": (I32, [VP, VP, U32, U32, VP, U32, U32, VP, VP]),
    "bvhgb_trace_image": (I32, [VP, U32, U32, VP, VP, C.POINTER(Camera), C.POINTER(TraceConfig), VP, VP, VP]),
    "bvhgb_trace_rays": (I32, [VP, U32, U32, VP, VP, VP, VP, U32, C.POINTER(TraceConfig), VP, VP]),
    "bvhgb_trace_bounce": (I32, [VP, U32, U32, VP, VP, C.POINTER(Camera), C.POINTER(TraceConfig), U64, F32, VP, VP,
                                 VP, VP, VP]),
    "bvhgb_trace_read_errors": (I32, [C.POINTER(U32), I32]),
    "bvhgb_generate_rays": (I32, [VP, C.POINTER(Camera), VP]),
    "bvhgb_trace_ray_image": (I32, [VP, U32, U32, VP, VP, VP, U32, C.POINTER(TraceConfig), I32, VP, VP, VP]),
    "bvhgb_tracer_create": (I32, [U32, C.POINTER(VP)]),
    "bvhgb_tracer_destroy": (I32, [VP]),
    "bvhgb_tracer_update": (I32, [VP, VP, U32, U32, VP]),
    "bvhgb_tracer_trace_image": (I32, [VP, VP, VP, C.POINTER(Camera), C.POINTER(TraceConfig), VP, VP, VP]),
    "bvhgb_tracer_trace_rays": (I32, [VP, VP, VP, VP, VP, U32, C.POINTER(TraceConfig), VP, VP]),
    "bvhgb_tracer_trace_bounce": (I32, [VP, VP, VP, C.POINTER(Camera), C.POINTER(TraceConfig), U64, F32, VP, VP, VP,
                                        VP, VP]),
    "bvhgb_copy_mesh_to_gpu": (I32, [VP, U32, VP, U32, VP, U32, C.POINTER(MeshRaw)]),
    "bvhgb_copy_mesh_to_host": (I32, [C.POINTER(MeshRaw), VP, VP, VP]),
    "bvhgb_copy_bvh_to_gpu": (I32, [VP, U32, U32, C.c_uint16, C.POINTER(BvhPointer)]),
    "bvhgb_allocate_bvh": (I32, [C.POINTER(BvhPointer), U32]),
    "bvhgb_copy_bvh_to_host": (I32, [C.POINTER(BvhPointer), VP, U32, C.POINTER(U32), C.POINTER(C.c_uint16)]),
    "bvhgb_free_bvh": (I32, [C.POINTER(BvhPointer)]),
    "bvhgb_free_mesh": (I32, [C.POINTER(MeshRaw)]),
    "bvhgb_fix_levels_host": (I32, [VP, U32, U32, C.POINTER(C.c_uint16)]),
    "bvhgb_device_sync": (I32, []),
    "bvhgb_reset_device": (I32, []),
}

_lib = None


def load(path: os.PathLike | None = None):
    """Load libbvhgb.so (building it first only if it has never been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        from . import _build
        _build.build()
    if not p.exists():
        raise RuntimeError(f"{p} is missing: the CUDA library has not been built")
    lib = C.CDLL(str(p))
    for name, (res, args) in PROTOS.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, where: str):
    if status != 0:
        detail = load().bvhgb_last_error().decode(errors="replace")
        raise BvhgbError(status, where, detail)
