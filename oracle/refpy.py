"""ctypes bindings of oracle/_ref/libref.so: the reference's own CPU command classes (test
infrastructure only). lib() returns None where the reference's sources are absent (the library is
built from them by oracle/build_ref.py), and callers skip."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build_ref
from .pyoracle import NODE_DTYPE

_lib = None
_tried = False


def lib():
    global _lib, _tried
    if not _tried:
        _tried = True
        path = build_ref.build()
        if path is not None:
            _lib = C.CDLL(str(path))
            _lib.ref_calc_sah.restype = C.c_float
            _lib.ref_fix_levels.restype = C.c_uint32
            _lib.ref_trace.restype = C.c_int64
            _lib.ref_build.restype = C.c_int64
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _v3(x):
    return (C.c_float * 3)(*map(float, x))


def bittner13(nodes, iters, batch_percent=1.0, root=0, threads=1):
    """Bittner13::runImpl + teardown on a copy; returns (nodes, SAH trace [iters + 1], status)."""
    nodes = np.ascontiguousarray(nodes, NODE_DTYPE).copy()
    trace = np.zeros(iters + 1, np.float32)
    st = lib().ref_bittner13(_p(nodes), C.c_uint32(nodes.shape[0]), C.c_uint32(root), C.c_uint32(iters),
                             C.c_float(batch_percent), C.c_int(threads), _p(trace))
    return nodes, trace, st


def bittner13par(nodes, iters, num_chunks=32, batch_percent=1.0, offset_access=False, alt_find_node=False,
                 alt_queue=16, root=0, threads=1):
    """Bittner13Par setup/runImpl/teardown on a copy; returns (nodes, SAH trace, skipped, total, status)."""
    nodes = np.ascontiguousarray(nodes, NODE_DTYPE).copy()
    trace = np.zeros(iters + 1, np.float32)
    skipped, total = C.c_uint32(), C.c_uint32()
    st = lib().ref_bittner13par(_p(nodes), C.c_uint32(nodes.shape[0]), C.c_uint32(root), C.c_uint32(iters),
                                C.c_float(batch_percent), C.c_uint32(num_chunks), C.c_int(int(offset_access)),
                                C.c_int(int(alt_find_node)), C.c_uint32(alt_queue), C.c_int(threads), _p(trace),
                                C.byref(skipped), C.byref(total))
    return nodes, trace, skipped.value, total.value, st


def calc_sah(nodes, root=0, threads=1):
    nodes = np.ascontiguousarray(nodes, NODE_DTYPE)
    return lib().ref_calc_sah(_p(nodes), C.c_uint32(nodes.shape[0]), C.c_uint32(root), C.c_int(threads))


def fix_levels(nodes, root=0):
    """BVH::fixLevels in place; returns the maximum level."""
    assert nodes.flags.c_contiguous and nodes.dtype == NODE_DTYPE
    return lib().ref_fix_levels(_p(nodes), C.c_uint32(nodes.shape[0]), C.c_uint32(root))


def camera_rays(pos, lookat, up, fov, width, height, threads=1):
    org = np.zeros((width * height, 3), np.float32)
    dirs = np.zeros((width * height, 3), np.float32)
    lib().ref_camera_rays(_v3(pos), _v3(lookat), _v3(up), C.c_float(fov), C.c_uint32(width), C.c_uint32(height),
                          C.c_int(threads), _p(org), _p(dirs))
    return org, dirs


def trace(nodes, vert, faces, cam, light=(2.0, 2.0, 2.0), brute=False, root=0, threads=1):
    """One camera image through CPUTracer (or BruteForceTracer); returns (grey, intCount, hit, ns)."""
    pos, lookat, up, fov, w, h = cam
    nodes = np.ascontiguousarray(nodes, NODE_DTYPE)
    vert = np.ascontiguousarray(vert, np.float32)
    faces = np.ascontiguousarray(faces, np.uint32)
    grey = np.zeros(w * h, np.uint8)
    cnt = np.zeros(w * h, np.uint32)
    hit = np.zeros(w * h, np.uint8)
    ns = lib().ref_trace(C.c_int(int(brute)), _p(nodes), C.c_uint32(nodes.shape[0]), C.c_uint32(root), _p(vert),
                         C.c_uint32(vert.shape[0]), _p(faces), C.c_uint32(faces.shape[0]), _v3(pos), _v3(lookat),
                         _v3(up), C.c_float(fov), C.c_uint32(w), C.c_uint32(h), _v3(light), C.c_int(threads),
                         _p(grey), _p(cnt), _p(hit))
    if ns < 0:
        raise RuntimeError("reference tracer failed")
    return grey, cnt, hit.astype(bool), ns


def build(vert, faces, which="median", threads=1):
    """Median or Wald07 top-down build; returns (nodes, root)."""
    vert = np.ascontiguousarray(vert, np.float32)
    faces = np.ascontiguousarray(faces, np.uint32)
    cap = 2 * faces.shape[0]
    nodes = np.zeros(cap, NODE_DTYPE)
    root = C.c_uint32()
    n = lib().ref_build(C.c_int(0 if which == "median" else 1), _p(vert), C.c_uint32(vert.shape[0]), _p(faces),
                        C.c_uint32(faces.shape[0]), C.c_int(threads), _p(nodes), C.c_uint32(cap), C.byref(root))
    if n < 0:
        raise RuntimeError("reference build failed")
    return nodes[:n].copy(), root.value
