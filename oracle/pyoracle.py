"""ctypes bindings of the CPU oracle (test infrastructure only; never used by the product path)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build_oracle

NODE_DTYPE = np.dtype([
    ("mn", "<f4", (3,)), ("mx", "<f4", (3,)), ("parent", "<u4"), ("left", "<u4"), ("right", "<u4"),
    ("isLeafFlag", "<u2"), ("isLeft", "<u2"), ("level", "<u2"), ("pad", "<u2"), ("surfaceArea", "<f4"),
])
assert NODE_DTYPE.itemsize == 48
HIT_DTYPE = np.dtype([("prim", "<u4"), ("t", "<f4")])

REFCOMPAT, KARRAS = 0, 1
_lib = None


class Aabb(C.Structure):
    _fields_ = [("mn", C.c_float * 3), ("mx", C.c_float * 3)]


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("lookat", C.c_float * 3), ("up", C.c_float * 3), ("fov", C.c_float),
                ("width", C.c_uint32), ("height", C.c_uint32)]


class Bn13Cfg(C.Structure):
    _fields_ = [("num_chunks", C.c_uint32), ("batch_percent", C.c_float), ("offset_access", C.c_uint32),
                ("heap_cap", C.c_uint32), ("search_mode", C.c_uint32), ("conflict_rule", C.c_uint32),
                ("std_select", C.c_uint32)]


class Bn13Stats(C.Structure):
    _fields_ = [("items", C.c_uint64), ("applied", C.c_uint64), ("skipped_conflict", C.c_uint64),
                ("skipped_invalid", C.c_uint64), ("heap_overflow", C.c_uint64), ("nodes_visited", C.c_uint64)]


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build_oracle.build()))
        _lib.orc_sah.restype = C.c_double
        _lib.orc_surface_area.restype = C.c_float
        _lib.orc_inefficiency.restype = C.c_float
        _lib.orc_adler32.restype = C.c_uint32
        _lib.orc_fix_levels.restype = C.c_uint32
        _lib.orc_shade.restype = C.c_uint8
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def tri_data(vert, faces):
    vert, faces = _f32(vert), _u32(faces)
    n = faces.shape[0]
    box = np.zeros((n, 6), np.float32)
    cen = np.zeros((n, 3), np.float32)
    scene = Aabb()
    lib().orc_tri_data(_p(vert), _p(faces), C.c_uint32(n), _p(box), _p(cen), C.byref(scene))
    return box, cen, np.array(list(scene.mn) + list(scene.mx), np.float32)


def morton(centroids, scene, bits=30):
    cen = _f32(centroids)
    n = cen.shape[0]
    sc = Aabb((C.c_float * 3)(*scene[:3]), (C.c_float * 3)(*scene[3:]))
    off = (C.c_float * 3)()
    scale = (C.c_float * 3)()
    lib().orc_morton_params(C.byref(sc), off, scale)
    if bits == 30:
        out = np.zeros(n, np.uint32)
        lib().orc_morton30(_p(cen), C.c_uint32(n), off, scale, _p(out))
    else:
        out = np.zeros(n, np.uint64)
        lib().orc_morton63(_p(cen), C.c_uint32(n), off, scale, _p(out))
    return out


def sort_pairs(keys):
    keys = np.ascontiguousarray(keys)
    n = keys.shape[0]
    ko = np.zeros_like(keys)
    vo = np.zeros(n, np.uint32)
    if keys.dtype == np.uint32:
        lib().orc_sort_pairs32(_p(keys), C.c_uint32(n), _p(ko), _p(vo))
    else:
        lib().orc_sort_pairs64(_p(np.ascontiguousarray(keys, np.uint64)), C.c_uint32(n), _p(ko), _p(vo))
    return ko, vo


def lbvh_build(vert, faces, bits=30, mode=REFCOMPAT):
    vert, faces = _f32(vert), _u32(faces)
    n = faces.shape[0]
    nodes = np.zeros(max(2 * n - 1, 0), NODE_DTYPE)
    keys = np.zeros(n, np.uint32 if bits == 30 else np.uint64)
    idx = np.zeros(n, np.uint32)
    r = lib().orc_lbvh_build(_p(vert), _p(faces), C.c_uint32(n), C.c_int(bits), C.c_int(mode), _p(nodes),
                             _p(keys), _p(idx))
    if r != 0:
        raise ValueError("orc_lbvh_build failed")
    return nodes, keys, idx


def sah(nodes, root=0):
    nodes = np.ascontiguousarray(nodes)
    return lib().orc_sah(_p(nodes), C.c_uint32(nodes.shape[0]), C.c_uint32(root))


def fix_levels(nodes, root=0):
    return lib().orc_fix_levels(_p(nodes), C.c_uint32(nodes.shape[0]), C.c_uint32(root))


def validate(nodes, vert=None, faces=None, root=0, check_levels=False):
    errs = (C.c_uint32 * 5)()
    nf = 0 if faces is None else faces.shape[0]
    vert = None if vert is None else _f32(vert)
    faces = None if faces is None else _u32(faces)
    lib().orc_validate(_p(np.ascontiguousarray(nodes)), C.c_uint32(nodes.shape[0]), C.c_uint32(root), _p(vert),
                       _p(faces), C.c_uint32(nf), C.c_int(int(check_levels)), errs)
    return list(errs)


def bittner_seq(nodes, iters, batch_percent=1.0, root=0):
    nodes = np.ascontiguousarray(nodes).copy()
    r = C.c_uint32(root)
    trace = np.zeros(iters + 1, np.float64)
    lib().orc_bittner_seq(_p(nodes), C.c_uint32(nodes.shape[0]), C.byref(r), C.c_uint32(iters),
                          C.c_float(batch_percent), _p(trace))
    return nodes, r.value, trace


def bittner_chunked(nodes, iters, num_chunks=32, batch_percent=1.0, offset_access=False, heap_cap=4096, root=0,
                    search_mode=0, conflict_rule=0, std_select=0):
    """search_mode 0: batched best-first search (GPU default); 1: the reference's heap order.
    conflict_rule 0: lowest batch rank claims (GPU kernels); 1: Bittner13Par's first-come rule.
    std_select 0: stable inefficiency order (GPU kernels); 1: the reference CPU optimizers' order."""
    nodes = np.ascontiguousarray(nodes).copy()
    trace = np.zeros(iters + 1, np.float64)
    cfg = Bn13Cfg(num_chunks, batch_percent, int(offset_access), heap_cap, search_mode, conflict_rule, std_select)
    st = Bn13Stats()
    lib().orc_bittner_chunked(_p(nodes), C.c_uint32(nodes.shape[0]), C.c_uint32(root), C.c_uint32(iters),
                              C.byref(cfg), _p(trace), C.byref(st))
    stats = {k: getattr(st, k) for k, _ in Bn13Stats._fields_}
    return nodes, trace, stats


def bittner_chunked_until(nodes, max_iters, stop_sah, root=0, **cfg):
    """Chunked iterations in place until the SAH is <= stop_sah (or max_iters); returns
    (iterations run, SAH trace, per-iteration wall ms without the SAH evaluations, stats)."""
    assert nodes.flags.c_contiguous
    trace = np.zeros(max_iters + 1, np.float64)
    ms = np.zeros(max(max_iters, 1), np.float64)
    st = Bn13Stats()
    done = C.c_uint32()
    c = _cfg(**cfg)
    lib().orc_bittner_chunked_until(_p(nodes), C.c_uint32(nodes.shape[0]), C.c_uint32(root), C.c_uint32(max_iters),
                                    C.byref(c), C.c_double(stop_sah), _p(trace), _p(ms), C.byref(st), C.byref(done))
    k = done.value
    return k, trace[: k + 1].copy(), ms[:k].copy(), {f: getattr(st, f) for f, _ in Bn13Stats._fields_}


def camera_rays(pos, lookat, up, fov, width, height):
    cam = Camera((C.c_float * 3)(*pos), (C.c_float * 3)(*lookat), (C.c_float * 3)(*up), fov, width, height)
    org = np.zeros((height * width, 3), np.float32)
    dirs = np.zeros((height * width, 3), np.float32)
    lib().orc_camera_rays(C.byref(cam), _p(org), _p(dirs))
    return org, dirs


def ray_tri(org, d, v0, v1, v2, tmin=0.0, tmax=np.inf, cull=False):
    t = C.c_float()
    a = [(C.c_float * 3)(*map(float, x)) for x in (org, d, v0, v1, v2)]
    hit = lib().orc_ray_tri(a[0], a[1], a[2], a[3], a[4], C.c_float(tmin), C.c_float(tmax), C.c_int(int(cull)),
                            C.byref(t))
    return bool(hit), t.value


def trace_brute(org, dirs, vert, faces, tmin=0.0, tmax=np.inf, cull=False):
    org, dirs, vert, faces = _f32(org), _f32(dirs), _f32(vert), _u32(faces)
    hits = np.zeros(org.shape[0], HIT_DTYPE)
    lib().orc_trace_brute(_p(org), _p(dirs), C.c_uint32(org.shape[0]), _p(vert), _p(faces), C.c_uint32(faces.shape[0]),
                          C.c_float(tmin), C.c_float(tmax), C.c_int(int(cull)), _p(hits))
    return hits


def trace_bvh(org, dirs, nodes, vert, faces, root=0, tmin=0.0, tmax=np.inf, cull=False):
    org, dirs, vert, faces = _f32(org), _f32(dirs), _f32(vert), _u32(faces)
    hits = np.zeros(org.shape[0], HIT_DTYPE)
    lib().orc_trace_bvh(_p(org), _p(dirs), C.c_uint32(org.shape[0]), _p(np.ascontiguousarray(nodes)),
                        C.c_uint32(root), _p(vert), _p(faces), C.c_float(tmin), C.c_float(tmax), C.c_int(int(cull)),
                        _p(hits))
    return hits


def trace_cpu_reference(org, dirs, nodes, vert, faces, root=0):
    org, dirs, vert, faces = _f32(org), _f32(dirs), _f32(vert), _u32(faces)
    hits = np.zeros(org.shape[0], HIT_DTYPE)
    cnt = np.zeros(org.shape[0], np.uint16)
    lib().orc_trace_cpu_reference(_p(org), _p(dirs), C.c_uint32(org.shape[0]), _p(np.ascontiguousarray(nodes)),
                                  C.c_uint32(root), _p(vert), _p(faces), _p(hits), _p(cnt))
    return hits, cnt


def shade(org, d, t, v1, v2, v3, light=(2.0, 2.0, 2.0)):
    a = [(C.c_float * 3)(*map(float, x)) for x in (org, d)]
    b = [(C.c_float * 3)(*map(float, x)) for x in (v1, v2, v3, light)]
    return lib().orc_shade(a[0], a[1], C.c_float(t), b[0], b[1], b[2], b[3])


def adler32(data: bytes) -> int:
    buf = np.frombuffer(data, np.uint8)
    return lib().orc_adler32(_p(buf), C.c_size_t(len(data)))


def num_threads() -> int:
    return lib().orc_num_threads()


def set_threads(n: int):
    lib().orc_set_threads(C.c_int(n))


def _cfg(num_chunks=32, batch_percent=1.0, offset_access=False, heap_cap=4096, search_mode=0, conflict_rule=0,
         std_select=0):
    return Bn13Cfg(num_chunks, batch_percent, int(offset_access), heap_cap, search_mode, conflict_rule, std_select)


def bittner_iteration_ordered(nodes, order, root=0, **cfg):
    """One chunked iteration in place with the given batch order; returns the stats dict."""
    assert nodes.flags.c_contiguous
    order = _u32(order)
    st = Bn13Stats()
    c = _cfg(**cfg)
    lib().orc_bittner_iteration_ordered(_p(nodes), C.c_uint32(nodes.shape[0]), C.c_uint32(root), _p(order),
                                        C.c_uint32(order.shape[0]), C.byref(c), C.byref(st))
    return {k: getattr(st, k) for k, _ in Bn13Stats._fields_}


LR_FEATURES = 24


def lr_features(nodes, root=0):
    """(features [n_inner, 24] float32, inner node ids ascending)."""
    nodes = np.ascontiguousarray(nodes)
    n = nodes.shape[0]
    feat = np.zeros((n, LR_FEATURES), np.float32)
    inner = np.zeros(n, np.uint32)
    lib().orc_lr_features.restype = C.c_uint32
    m = lib().orc_lr_features(_p(nodes), C.c_uint32(n), C.c_uint32(root), _p(feat), _p(inner))
    return feat[:m].copy(), inner[:m].copy()


def lr_inv_log2_leaves(n_leaves):
    lib().orc_lr_inv_log2_leaves.restype = C.c_float
    return lib().orc_lr_inv_log2_leaves(C.c_uint32(n_leaves))


def bn13_gains(nodes, cand, root=0):
    """Isolated realised SAH reduction of reinserting each candidate alone (units of root SA)."""
    nodes = np.ascontiguousarray(nodes)
    cand = _u32(cand)
    gain = np.zeros(cand.shape[0], np.float32)
    ok = np.zeros(cand.shape[0], np.uint8)
    lib().orc_bn13_gains(_p(nodes), C.c_uint32(nodes.shape[0]), C.c_uint32(root), _p(cand), C.c_uint32(cand.shape[0]),
                         _p(gain), _p(ok))
    return gain, ok.astype(bool)
