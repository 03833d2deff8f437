"""Python face of the C ABI over torch CUDA tensors (device memory and streams only).

Each class mirrors one of the reference's commands / C functions and calls straight into
libbvhgb.so; device buffers are torch tensors, node arrays are int32 tensors of shape
(numNodes, 12) holding the 48-byte BVHNode records.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import native
from .native import (Aabb, BatchConfig, BatchTuneReport, BvhgbError, Bn13Config, Bn13Stats, Camera, HIT_DTYPE,
                     LbvhConfig, NODE_DTYPE, PIXEL_DTYPE,
                     TraceConfig, check, load)

REFCOMPAT, KARRAS = 0, 1
TOPOLOGY = {"refCompat": REFCOMPAT, "karras": KARRAS, REFCOMPAT: REFCOMPAT, KARRAS: KARRAS}


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _dev_f32(a):
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda", dtype=torch.float32).contiguous()
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _dev_u32(a):
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda", dtype=torch.int32).contiguous()
    return torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda()


def nodes_to_numpy(nodes: torch.Tensor) -> np.ndarray:
    return nodes.detach().cpu().contiguous().numpy().view(NODE_DTYPE).reshape(-1)


def nodes_from_numpy(arr: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(arr).view(np.int32).reshape(-1, 12).copy()).cuda()


def empty_nodes(n_nodes: int) -> torch.Tensor:
    return torch.empty((max(n_nodes, 1), 12), dtype=torch.int32, device="cuda")


class LBVH:
    """The `LBVH` command (lib/builder/LBVH.cpp:28-55) over a device-resident mesh."""

    def __init__(self, max_faces: int, morton_bits: int = 30, topology="refCompat"):
        self.lib = load()
        self.max_faces = int(max_faces)
        self.cfg = LbvhConfig(int(morton_bits), TOPOLOGY[topology])
        ws = C.c_void_p()
        check(self.lib.bvhgb_lbvh_create(self.max_faces, C.byref(self.cfg), C.byref(ws)), "bvhgb_lbvh_create")
        self.ws = ws

    def close(self):
        if self.ws:
            self.lib.bvhgb_lbvh_destroy(self.ws)
            self.ws = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build(self, vert, faces, nodes=None, stream=None) -> torch.Tensor:
        v, f = _dev_f32(vert), _dev_u32(faces)
        n = f.shape[0]
        if nodes is None:
            nodes = empty_nodes(2 * n - 1)
        check(self.lib.bvhgb_lbvh_build(self.ws, _ptr(v), _ptr(f), n, _ptr(nodes), _stream(stream)), "bvhgb_lbvh_build")
        return nodes

    # phases (LBVH_initTriData, LBVH_calcMortonCodes, LBVH_sortMortonCodes, LBVH_buildBVHTree)
    def init_tri_data(self, vert, faces, stream=None):
        check(self.lib.bvhgb_lbvh_init_tri_data(self.ws, _ptr(vert), _ptr(faces), faces.shape[0], _stream(stream)),
              "init_tri_data")

    def calc_morton(self, vert, faces, stream=None):
        check(self.lib.bvhgb_lbvh_calc_morton(self.ws, _ptr(vert), _ptr(faces), faces.shape[0], _stream(stream)),
              "calc_morton")

    def sort(self, n, stream=None):
        check(self.lib.bvhgb_lbvh_sort(self.ws, n, _stream(stream)), "sort")

    def build_tree(self, vert, faces, nodes, stream=None):
        check(self.lib.bvhgb_lbvh_build_tree(self.ws, _ptr(vert), _ptr(faces), faces.shape[0], _ptr(nodes),
                                             _stream(stream)), "build_tree")

    def scene_box(self, stream=None) -> np.ndarray:
        a = Aabb()
        check(self.lib.bvhgb_lbvh_read_scene_box(self.ws, C.byref(a), _stream(stream)), "read_scene_box")
        return np.array(list(a.mn) + list(a.mx), np.float32)

    def errors(self, stream=None) -> int:
        v = C.c_uint32()
        check(self.lib.bvhgb_lbvh_read_errors(self.ws, C.byref(v), _stream(stream)), "read_errors")
        return v.value

    def keys(self, n, sorted_: bool, stream=None):
        k = np.zeros(n, np.uint32 if self.cfg.mortonBits == 30 else np.uint64)
        idx = np.zeros(n, np.uint32)
        check(self.lib.bvhgb_lbvh_read_keys(self.ws, int(sorted_), k.ctypes.data_as(C.c_void_p),
                                            idx.ctypes.data_as(C.c_void_p), n, _stream(stream)), "read_keys")
        return k, idx


def select_smallest_pairs(keys: torch.Tensor, vals: torch.Tensor, k: int, stream=None) -> torch.Tensor:
    """Values of the k smallest keys (int32 tensors, keys read as unsigned) in stable ascending order:
    the first k values of radix_sort_pairs(keys, vals)."""
    lib = load()
    n = keys.shape[0]
    need = C.c_size_t(0)
    check(lib.bvhgb_select_smallest_pairs(None, C.byref(need), None, None, None, n, k, None), "select size")
    temp = torch.empty(max(need.value, 1), dtype=torch.uint8, device="cuda")
    out = torch.empty(k, dtype=vals.dtype, device="cuda")
    check(lib.bvhgb_select_smallest_pairs(_ptr(temp), C.byref(need), _ptr(keys), _ptr(vals), _ptr(out), n, k,
                                          _stream(stream)), "bvhgb_select_smallest_pairs")
    return out


def radix_sort_pairs(keys: torch.Tensor, vals: torch.Tensor, begin_bit=0, end_bit=None, stream=None):
    """Stable ascending sort of (key, value) pairs; keys int32/int64 tensors read as unsigned."""
    lib = load()
    kb = keys.element_size()
    end_bit = 8 * kb if end_bit is None else end_bit
    n = keys.shape[0]
    need = C.c_size_t(0)
    check(lib.bvhgb_radix_sort_pairs(None, C.byref(need), None, None, None, None, n, kb, begin_bit, end_bit, None),
          "sort size")
    temp = torch.empty(max(need.value, 1), dtype=torch.uint8, device="cuda")
    ko = torch.empty_like(keys)
    vo = torch.empty_like(vals)
    check(lib.bvhgb_radix_sort_pairs(_ptr(temp), C.byref(need), _ptr(keys), _ptr(ko), _ptr(vals), _ptr(vo), n, kb,
                                     begin_bit, end_bit, _stream(stream)), "bvhgb_radix_sort_pairs")
    return ko, vo


def sort_default_tile(tile_keys: int = 0) -> int:
    """Sets the onesweep tile (2048, 4096 or 8192 keys per CTA) of the sorts that are not given one
    (LBVH build, optimizer selection) and returns the previous setting; 0 only reads it."""
    prev = C.c_uint32()
    check(load().bvhgb_sort_set_default_tile(int(tile_keys), C.byref(prev)), "bvhgb_sort_set_default_tile")
    return prev.value


def calc_sah(nodes: torch.Tensor, root: int = 0, num_nodes=None, stream=None) -> float:
    out = C.c_double()
    n = nodes.shape[0] if num_nodes is None else num_nodes
    check(load().bvhgb_calc_sah(_ptr(nodes), n, root, C.byref(out), _stream(stream)), "bvhgb_calc_sah")
    return out.value


class Bittner13GPU:
    """The `bittner13GPU` command (lib/builder/Bittner13GPU.cpp:78-133)."""

    def __init__(self, nodes: torch.Tensor, root: int = 0, num_chunks=32, block_size=128, batch_percent=1.0,
                 offset_access=False, heap_capacity=4096, num_nodes=None, profile=False, search_mode=0, stream=None):
        self.lib = load()
        self.cfg = Bn13Config(num_chunks, block_size, batch_percent, int(offset_access), heap_capacity, int(profile),
                              int(search_mode))
        ws = C.c_void_p()
        n = nodes.shape[0] if num_nodes is None else num_nodes
        check(self.lib.bvhgb_bn13_create(_ptr(nodes), n, root, C.byref(self.cfg), C.byref(ws), _stream(stream)),
              "bvhgb_bn13_create")
        self.ws = ws
        self.nodes = nodes

    def close(self):
        if self.ws:
            self.lib.bvhgb_bn13_destroy(self.ws)
            self.ws = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def batch_size(self) -> int:
        return self.lib.bvhgb_bn13_batch_size(self.ws)

    @property
    def launches_per_iteration(self) -> int:
        return self.lib.bvhgb_bn13_launches_per_iteration(self.ws)

    def search_time(self):
        """(ms, launches) of the reinsertion-search kernel in the last iteration (profile=True)."""
        ms = C.c_float()
        n = C.c_uint32()
        check(self.lib.bvhgb_bn13_search_time(self.ws, C.byref(ms), C.byref(n)), "bvhgb_bn13_search_time")
        return ms.value, n.value

    def step(self, stream=None):
        check(self.lib.bvhgb_bn13_step(self.ws, _ptr(self.nodes), _stream(stream)), "bvhgb_bn13_step")

    def run(self, iterations: int, stream=None):
        check(self.lib.bvhgb_bn13_run(self.ws, _ptr(self.nodes), iterations, _stream(stream)), "bvhgb_bn13_run")

    def stats(self, stream=None) -> dict:
        st = Bn13Stats()
        check(self.lib.bvhgb_bn13_get_stats(self.ws, C.byref(st), _stream(stream)), "bvhgb_bn13_get_stats")
        return {k: getattr(st, k) for k, _ in Bn13Stats._fields_}

    @property
    def num_inner(self) -> int:
        n = C.c_uint32()
        check(self.lib.bvhgb_bn13_read_inner(self.ws, None, 0, C.byref(n), None), "bvhgb_bn13_read_inner")
        return n.value

    def inner_nodes(self, stream=None) -> torch.Tensor:
        """The ascending inner-node list (int32, device copy)."""
        n = self.num_inner
        out = torch.empty(n, dtype=torch.int32, device="cuda")
        check(self.lib.bvhgb_bn13_read_inner(self.ws, _ptr(out), n, None, _stream(stream)), "bvhgb_bn13_read_inner")
        return out

    def selection(self, stream=None) -> torch.Tensor:
        """Node order of the most recent selection (int32, device copy, batch position order): the
        first min(batch_size, num_inner) entries, the ones the chunks process."""
        out = torch.empty(min(self.batch_size, self.num_inner), dtype=torch.int32, device="cuda")
        check(self.lib.bvhgb_bn13_read_selection(self.ws, _ptr(out), out.shape[0], _stream(stream)),
              "bvhgb_bn13_read_selection")
        return out

    def set_selection(self, order: torch.Tensor, stream=None):
        """Use 'order' (numInner node ids, batch position order) for the following chunk() calls."""
        order = order.to(device="cuda", dtype=torch.int32).contiguous()
        check(self.lib.bvhgb_bn13_set_selection(self.ws, _ptr(order), order.shape[0], _stream(stream)),
              "bvhgb_bn13_set_selection")

    def select(self, stream=None):
        check(self.lib.bvhgb_bn13_select_nodes(self.ws, _ptr(self.nodes), _stream(stream)), "bvhgb_bn13_select_nodes")

    def chunk(self, c: int, stream=None):
        check(self.lib.bvhgb_bn13_chunk(self.ws, _ptr(self.nodes), c, _stream(stream)), "bvhgb_bn13_chunk")

    def gains(self, cand: torch.Tensor, with_target=False, stream=None):
        """Realised SAH reduction of reinserting each candidate alone (and the training target)."""
        cand = cand.to(device="cuda", dtype=torch.int32).contiguous()
        gain = torch.empty(cand.shape[0], dtype=torch.float32, device="cuda")
        tgt = torch.empty_like(gain) if with_target else None
        check(self.lib.bvhgb_bn13_gains(self.ws, _ptr(self.nodes), _ptr(cand), cand.shape[0], _ptr(gain), _ptr(tgt),
                                        _stream(stream)), "bvhgb_bn13_gains")
        return (gain, tgt) if with_target else gain

    def set_scorer(self, scorer: "Mlp | None", plain_every: int = 2):
        """Learned selection with 'scorer' (kept referenced here); every plain_every-th iteration still
        selects by the inefficiency (2 = alternate, 0 = scorer only). None restores the plain measure."""
        check(self.lib.bvhgb_bn13_set_scorer(self.ws, scorer.handle if scorer is not None else None, plain_every),
              "bvhgb_bn13_set_scorer")
        self._scorer = scorer

    def set_tail_packing(self, climbs_per_warp: int = 0):
        """Climbs per warp of the chunk tail (1..32, 0 = automatic); the trees do not depend on it."""
        check(self.lib.bvhgb_bn13_set_tail_packing(self.ws, climbs_per_warp), "bvhgb_bn13_set_tail_packing")

    @property
    def iteration(self) -> int:
        return self.lib.bvhgb_bn13_iteration(self.ws)

    @iteration.setter
    def iteration(self, it: int):
        check(self.lib.bvhgb_bn13_set_iteration(self.ws, it), "bvhgb_bn13_set_iteration")


MLP_PARAMS = 5825
LR_FEATURES = 24


class Mlp:
    """The learned reinsertion scorer (bvhgb_mlp_*): 24 -> 64 -> 64 -> 1 GELU, BF16 compute."""

    def __init__(self, seed: int = 0, params=None):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.bvhgb_mlp_create(seed, C.byref(h)), "bvhgb_mlp_create")
        self.handle = h
        if params is not None:
            self.set_params(params)

    def close(self):
        if self.handle:
            self.lib.bvhgb_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def save(self, path):
        """Raw little-endian float32 parameters (the `learnedScorer` file of the bittner13GPU command)."""
        self.params().astype("<f4").tofile(path)

    @classmethod
    def load(cls, path) -> "Mlp":
        return cls(params=np.fromfile(path, dtype="<f4"))

    def params(self) -> np.ndarray:
        out = np.zeros(MLP_PARAMS, np.float32)
        check(self.lib.bvhgb_mlp_get_params(self.handle, out.ctypes.data_as(C.c_void_p)), "bvhgb_mlp_get_params")
        return out

    def set_params(self, params):
        a = np.ascontiguousarray(params, dtype=np.float32)
        assert a.shape == (MLP_PARAMS,)
        check(self.lib.bvhgb_mlp_set_params(self.handle, a.ctypes.data_as(C.c_void_p)), "bvhgb_mlp_set_params")

    def forward(self, x: torch.Tensor, stream=None) -> torch.Tensor:
        """x: [n, 24] bfloat16 device rows -> float32 [n]."""
        x = x.contiguous()
        assert x.dtype == torch.bfloat16 and x.shape[1] == LR_FEATURES
        y = torch.empty(x.shape[0], dtype=torch.float32, device="cuda")
        check(self.lib.bvhgb_mlp_forward(self.handle, _ptr(x), x.shape[0], _ptr(y), _stream(stream)),
              "bvhgb_mlp_forward")
        return y

    def gradient(self, x: torch.Tensor, t: torch.Tensor, stream=None):
        """(gradient [5825] float32 numpy, loss) of the mean squared error over all rows."""
        x, t = x.contiguous(), t.to(torch.float32).contiguous()
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = C.c_float()
        check(self.lib.bvhgb_mlp_gradient(self.handle, _ptr(x), _ptr(t), x.shape[0], g.ctypes.data_as(C.c_void_p),
                                          C.byref(loss), _stream(stream)), "bvhgb_mlp_gradient")
        return g, loss.value

    def train(self, x: torch.Tensor, t: torch.Tensor, steps: int, batch=8192, lr=1e-3, weight_decay=1e-4, seed=0,
              stream=None, with_loss=True):
        x, t = x.contiguous(), t.to(torch.float32).contiguous()
        hist = np.zeros(max(steps, 1), np.float32) if with_loss else None
        check(self.lib.bvhgb_mlp_train(self.handle, _ptr(x), _ptr(t), x.shape[0], batch, steps, lr, weight_decay, seed,
                                       hist.ctypes.data_as(C.c_void_p) if hist is not None else None,
                                       _stream(stream)), "bvhgb_mlp_train")
        return hist[:steps] if hist is not None else None


class LrFeatures:
    """Feature rows of the learned scorer (bvhgb_lr_features_*)."""

    def __init__(self, max_nodes: int):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.bvhgb_lr_features_create(max_nodes, C.byref(h)), "bvhgb_lr_features_create")
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.bvhgb_lr_features_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __call__(self, nodes: torch.Tensor, inner: torch.Tensor, root=0, num_nodes=None, stream=None) -> torch.Tensor:
        n = nodes.shape[0] if num_nodes is None else num_nodes
        inner = inner.to(device="cuda", dtype=torch.int32).contiguous()
        x = torch.empty((inner.shape[0], LR_FEATURES), dtype=torch.bfloat16, device="cuda")
        num_leaves = n - inner.shape[0]
        check(self.lib.bvhgb_lr_features(self.handle, _ptr(nodes), n, root, _ptr(inner), inner.shape[0], num_leaves,
                                         _ptr(x), _stream(stream)), "bvhgb_lr_features")
        return x


def make_camera(pos, lookAt, up, fov, width, height) -> Camera:
    return Camera((C.c_float * 3)(*pos), (C.c_float * 3)(*lookAt), (C.c_float * 3)(*up), float(fov), int(width),
                  int(height))


def make_trace_config(light=(2.0, 2.0, 2.0), face_culling=False, tmin=0.0, tmax=float("inf"),
                      ray_bundles=False) -> TraceConfig:
    return TraceConfig((C.c_float * 3)(*light), int(face_culling), float(tmin), float(tmax), int(ray_bundles))


def trace_image(nodes, vert, faces, camera: dict, root=0, light=(2.0, 2.0, 2.0), face_culling=False, with_hits=True,
                num_nodes=None, ray_bundles=False, stream=None):
    """generateRays + tracerImage (CUDAKernels.cu:386-417): returns (pixels int32 [h*w], hits int64 [h*w] | None).
    ray_bundles: warps traverse as bundles (the reference's rayBundles); same hits."""
    cam = make_camera(**camera)
    cfg = make_trace_config(light, face_culling, ray_bundles=ray_bundles)
    npx = cam.width * cam.height
    img = torch.empty(npx, dtype=torch.int32, device="cuda")
    hits = torch.empty(npx, dtype=torch.int64, device="cuda") if with_hits else None
    n = nodes.shape[0] if num_nodes is None else num_nodes
    check(load().bvhgb_trace_image(_ptr(nodes), n, root, _ptr(vert), _ptr(faces), C.byref(cam), C.byref(cfg), _ptr(img),
                                   _ptr(hits), _stream(stream)), "bvhgb_trace_image")
    return img, hits


def trace_rays(nodes, vert, faces, org, dirs, root=0, tmin=0.0, tmax=float("inf"), face_culling=False, num_nodes=None,
               stream=None):
    cfg = make_trace_config((2.0, 2.0, 2.0), face_culling, tmin, tmax)
    o, d = _dev_f32(org), _dev_f32(dirs)
    hits = torch.empty(o.shape[0], dtype=torch.int64, device="cuda")
    n = nodes.shape[0] if num_nodes is None else num_nodes
    check(load().bvhgb_trace_rays(_ptr(nodes), n, root, _ptr(vert), _ptr(faces), _ptr(o), _ptr(d), o.shape[0],
                                  C.byref(cfg), _ptr(hits), _stream(stream)), "bvhgb_trace_rays")
    return hits


def trace_bounce(nodes, vert, faces, camera: dict, primary_hits, seed=1, offset=1e-4, root=0, with_rays=False,
                 num_nodes=None, stream=None):
    """One cosine-weighted bounce per primary hit; returns (hits int64 [h*w], org, dir | None)."""
    cam = make_camera(**camera)
    cfg = make_trace_config()
    npx = cam.width * cam.height
    out = torch.empty(npx, dtype=torch.int64, device="cuda")
    org = torch.empty((npx, 3), dtype=torch.float32, device="cuda") if with_rays else None
    dirs = torch.empty((npx, 3), dtype=torch.float32, device="cuda") if with_rays else None
    n = nodes.shape[0] if num_nodes is None else num_nodes
    check(load().bvhgb_trace_bounce(_ptr(nodes), n, root, _ptr(vert), _ptr(faces), C.byref(cam), C.byref(cfg), seed,
                                    offset, _ptr(primary_hits), _ptr(out), _ptr(org), _ptr(dirs), _stream(stream)),
          "bvhgb_trace_bounce")
    return out, org, dirs


class Tracer:
    """A tracer prepared for one tree (bvhgb_tracer_*): update() builds its traversal records (64 B
    per inner node), after which trace_image / trace_rays / trace_bounce give the same hits as the
    module functions with one record load per visit. The node tensor must not change between
    update() and the traces."""

    def __init__(self, max_nodes: int):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.bvhgb_tracer_create(int(max_nodes), C.byref(h)), "bvhgb_tracer_create")
        self.handle = h
        self.nodes = None

    def close(self):
        if self.handle:
            self.lib.bvhgb_tracer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update(self, nodes, root=0, num_nodes=None, stream=None):
        n = nodes.shape[0] if num_nodes is None else num_nodes
        check(self.lib.bvhgb_tracer_update(self.handle, _ptr(nodes), n, root, _stream(stream)), "bvhgb_tracer_update")
        self.nodes = nodes  # kept alive: the records point into it
        return self

    def trace_image(self, vert, faces, camera: dict, light=(2.0, 2.0, 2.0), face_culling=False, with_hits=True,
                    ray_bundles=False, stream=None):
        cam = make_camera(**camera)
        cfg = make_trace_config(light, face_culling, ray_bundles=ray_bundles)
        npx = cam.width * cam.height
        img = torch.empty(npx, dtype=torch.int32, device="cuda")
        hits = torch.empty(npx, dtype=torch.int64, device="cuda") if with_hits else None
        check(self.lib.bvhgb_tracer_trace_image(self.handle, _ptr(vert), _ptr(faces), C.byref(cam), C.byref(cfg),
                                                _ptr(img), _ptr(hits), _stream(stream)), "bvhgb_tracer_trace_image")
        return img, hits

    def trace_rays(self, vert, faces, org, dirs, tmin=0.0, tmax=float("inf"), face_culling=False, stream=None):
        cfg = make_trace_config((2.0, 2.0, 2.0), face_culling, tmin, tmax)
        o, d = _dev_f32(org), _dev_f32(dirs)
        hits = torch.empty(o.shape[0], dtype=torch.int64, device="cuda")
        check(self.lib.bvhgb_tracer_trace_rays(self.handle, _ptr(vert), _ptr(faces), _ptr(o), _ptr(d), o.shape[0],
                                               C.byref(cfg), _ptr(hits), _stream(stream)), "bvhgb_tracer_trace_rays")
        return hits

    def trace_bounce(self, vert, faces, camera: dict, primary_hits, seed=1, offset=1e-4, with_rays=False, stream=None):
        cam = make_camera(**camera)
        cfg = make_trace_config()
        npx = cam.width * cam.height
        out = torch.empty(npx, dtype=torch.int64, device="cuda")
        org = torch.empty((npx, 3), dtype=torch.float32, device="cuda") if with_rays else None
        dirs = torch.empty((npx, 3), dtype=torch.float32, device="cuda") if with_rays else None
        check(self.lib.bvhgb_tracer_trace_bounce(self.handle, _ptr(vert), _ptr(faces), C.byref(cam), C.byref(cfg), seed,
                                                 offset, _ptr(primary_hits), _ptr(out), _ptr(org), _ptr(dirs),
                                                 _stream(stream)), "bvhgb_tracer_trace_bounce")
        return out, org, dirs


def trace_errors(reset=True) -> int:
    v = C.c_uint32()
    check(load().bvhgb_trace_read_errors(C.byref(v), int(reset)), "bvhgb_trace_read_errors")
    return v.value


def hits_to_numpy(h: torch.Tensor) -> np.ndarray:
    return h.detach().cpu().numpy().view(HIT_DTYPE).reshape(-1)


def pixels_to_numpy(p: torch.Tensor) -> np.ndarray:
    return p.detach().cpu().numpy().view(PIXEL_DTYPE).reshape(-1)


class Batch:
    """Batched multi-mesh pipeline (bvhgb_batch_*): many meshes built, optimised and traced together.

    vert / faces are the meshes' vertices and faces concatenated (face vertex indices into the
    concatenated vertices); nodes holds every mesh's node array at its node offset."""

    def __init__(self, face_counts, topology="refCompat", num_chunks=32, batch_percent=1.0, sort_tile=8192,
                 refit_block=128, trace_block=128):
        self.lib = load()
        counts = np.ascontiguousarray(face_counts, dtype=np.uint32)
        self.num_meshes = int(counts.shape[0])
        cfg = BatchConfig(30, TOPOLOGY[topology], num_chunks, batch_percent, sort_tile, refit_block, trace_block)
        h = C.c_void_p()
        check(self.lib.bvhgb_batch_create(self.num_meshes, counts.ctypes.data_as(C.c_void_p), C.byref(cfg), C.byref(h)),
              "bvhgb_batch_create")
        self.ws = h
        fo = np.zeros(self.num_meshes + 1, np.uint32)
        no = np.zeros(self.num_meshes + 1, np.uint32)
        check(self.lib.bvhgb_batch_offsets(self.ws, fo.ctypes.data_as(C.c_void_p), no.ctypes.data_as(C.c_void_p)),
              "bvhgb_batch_offsets")
        self.face_offsets, self.node_offsets = fo, no

    def close(self):
        if self.ws:
            self.lib.bvhgb_batch_destroy(self.ws)
            self.ws = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def total_nodes(self) -> int:
        return int(self.node_offsets[-1])

    def empty_nodes(self) -> torch.Tensor:
        return empty_nodes(self.total_nodes)

    @property
    def config(self) -> dict:
        c = BatchConfig()
        check(self.lib.bvhgb_batch_get_config(self.ws, C.byref(c)), "bvhgb_batch_get_config")
        return {k: getattr(c, k) for k, _ in BatchConfig._fields_}

    def set_config(self, **kw):
        c = BatchConfig()
        check(self.lib.bvhgb_batch_get_config(self.ws, C.byref(c)), "bvhgb_batch_get_config")
        for k, v in kw.items():
            setattr(c, k, TOPOLOGY[v] if k == "topology" else v)
        check(self.lib.bvhgb_batch_set_config(self.ws, C.byref(c)), "bvhgb_batch_set_config")

    def build(self, vert, faces, nodes, stream=None):
        check(self.lib.bvhgb_batch_build(self.ws, _ptr(vert), _ptr(faces), _ptr(nodes), _stream(stream)),
              "bvhgb_batch_build")

    def optimize(self, nodes, iterations, stream=None):
        check(self.lib.bvhgb_batch_optimize(self.ws, _ptr(nodes), iterations, _stream(stream)), "bvhgb_batch_optimize")

    def trace_random(self, nodes, vert, faces, rays_per_mesh, seed=1, with_rays=False, stream=None):
        r = self.num_meshes * rays_per_mesh
        hits = torch.empty(r, dtype=torch.int64, device="cuda")
        org = torch.empty((r, 3), dtype=torch.float32, device="cuda") if with_rays else None
        dirs = torch.empty((r, 3), dtype=torch.float32, device="cuda") if with_rays else None
        check(self.lib.bvhgb_batch_trace_random(self.ws, _ptr(nodes), _ptr(vert), _ptr(faces), rays_per_mesh, seed,
                                                _ptr(hits), _ptr(org), _ptr(dirs), _stream(stream)),
              "bvhgb_batch_trace_random")
        return (hits, org, dirs) if with_rays else hits

    def run(self, vert, faces, nodes, iterations, rays_per_mesh, hits, seed=1, stream=None):
        check(self.lib.bvhgb_batch_run(self.ws, _ptr(vert), _ptr(faces), _ptr(nodes), iterations, rays_per_mesh, seed,
                                       _ptr(hits), _stream(stream)), "bvhgb_batch_run")

    def stats(self, stream=None):
        st = Bn13Stats()
        err = C.c_uint32()
        check(self.lib.bvhgb_batch_get_stats(self.ws, C.byref(st), C.byref(err), _stream(stream)),
              "bvhgb_batch_get_stats")
        return {k: getattr(st, k) for k, _ in Bn13Stats._fields_}, err.value

    def autotune(self, vert, faces, nodes, rays_per_mesh, hits, seed=1, stream=None) -> dict:
        rep = BatchTuneReport()
        check(self.lib.bvhgb_batch_autotune(self.ws, _ptr(vert), _ptr(faces), _ptr(nodes), rays_per_mesh, seed,
                                            _ptr(hits), C.byref(rep), _stream(stream)), "bvhgb_batch_autotune")
        chosen = {k: getattr(rep.chosen, k) for k, _ in BatchConfig._fields_}
        return {"sort_tile": dict(zip(list(rep.sortTileKeys), [round(v, 4) for v in rep.sortTileMs])),
                "refit_block": dict(zip(list(rep.refitBlock), [round(v, 4) for v in rep.refitBlockMs])),
                "trace_block": dict(zip(list(rep.traceBlock), [round(v, 4) for v in rep.traceBlockMs])),
                "chosen": chosen}

    def mesh_nodes(self, nodes: torch.Tensor, m: int) -> torch.Tensor:
        return nodes[int(self.node_offsets[m]): int(self.node_offsets[m + 1])]
