"""The allocation-free LBVH build, bvhgb_lbvh_build_static.

It exists for callers that cannot call cudaMalloc while they build (a per-frame rebuild in a render
or simulation loop, where an allocation synchronises the device; a host application whose device
memory all comes from its own pool). Its working memory is one file-scope device array shared by
every call, so the checks below run several calls in a row, each against the ordinary
(allocating) build of the same mesh, which must give the same bytes. This file is collected last
so that a run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from bvhtest_gb300 import scenes

pytestmark = pytest.mark.gpu

TOO_LARGE = 11
MAX_FACES = 262144  # BVHGB_STATIC_MAX_FACES in include/bvhgb.h


def _entry():
    from bvhtest_gb300 import native
    lib = native.load()
    fn = lib.bvhgb_lbvh_build_static
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(native.LbvhConfig), C.c_void_p, C.c_void_p]
    return fn, native


def _errors(native, cfg, stream):
    """Device error bits the last static build left in the shared array (0 = valid tree)."""
    fn = native.load().bvhgb_lbvh_static_read_errors
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(native.LbvhConfig), C.POINTER(C.c_uint32), C.c_void_p]
    flags = C.c_uint32(0xFFFFFFFF)
    assert fn(C.byref(cfg), C.byref(flags), stream) == 0
    return flags.value


def _mesh(n, seed):
    import torch
    vert, faces = scenes.uniform_soup(n, seed=seed)
    return torch.from_numpy(vert).cuda(), torch.from_numpy(faces.view(np.int32)).cuda()


def test_static_build_matches_allocating_build_on_consecutive_calls():
    import torch
    from bvhtest_gb300 import api
    build_static, native = _entry()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    # consecutive calls of different sizes and settings share the one scratch array
    for n, bits, topo, seed in ((200000, 30, 0, 5), (MAX_FACES, 63, 1, 6), (1000, 30, 1, 7), (1000, 30, 1, 7)):
        v, f = _mesh(n, seed)
        expected = api.LBVH(n, bits, topo).build(v, f)[: 2 * n - 1]
        out = torch.full((2 * n - 1, 12), -1, dtype=torch.int32, device="cuda")
        cfg = native.LbvhConfig(bits, topo)
        st = build_static(C.c_void_p(v.data_ptr()), C.c_void_p(f.data_ptr()), n, C.byref(cfg),
                          C.c_void_p(out.data_ptr()), stream)
        assert st == 0, native.load().bvhgb_last_error()
        assert _errors(native, cfg, stream) == 0, (n, bits, topo)
        torch.cuda.synchronize()
        assert torch.equal(out, expected), (n, bits, topo)


def test_static_build_rejects_sizes_above_its_maximum():
    import torch
    build_static, native = _entry()
    v, f = _mesh(MAX_FACES + 1, 8)
    out = torch.empty((2 * (MAX_FACES + 1) - 1, 12), dtype=torch.int32, device="cuda")
    cfg = native.LbvhConfig(30, 0)
    st = build_static(C.c_void_p(v.data_ptr()), C.c_void_p(f.data_ptr()), MAX_FACES + 1, C.byref(cfg),
                      C.c_void_p(out.data_ptr()), None)
    assert st == TOO_LARGE
