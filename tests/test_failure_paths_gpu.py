"""Failure paths on the GPU, made to happen without faulting or hanging anything.

* A bounded wait that runs out: the sort's decoupled look-back polls a predecessor tile's status
  word a bounded number of times (lib/builder/LBVH_CUDA.cu:185-193 is the sort it replaces; the
  reference's cub sort has no such bound). With the limit set to zero every tile that finds a
  predecessor still ranking gives up at once, raises the timeout bit, and scatters with the prefix
  it has, inside the arrays; the status reaches the host through bvhgb_lbvh_read_errors, and the
  context stays usable: the next build, with the limit restored, is byte-identical to a normal one.
  The timed-out sort's output is garbage by design and is never built into a tree.
* Allocation failure: the library's device allocations go through an injection point; making the
  Nth allocation of a create call fail must give OUT_OF_MEMORY (the reference's CUDA_RUN ... goto
  error, LBVH_CUDA.cu:29-39, Bittner13CUDA.cu:33-53), free what was allocated, and leave nothing
  allocated after the sweep.
"""
import ctypes as C

import numpy as np
import pytest

from bvhtest_gb300 import scenes

pytestmark = pytest.mark.gpu
OUT_OF_MEMORY = 10
TIMEOUT_BIT = 1


def _lib():
    from bvhtest_gb300 import native
    return native.load(), native


def test_lookback_timeout_is_reported_and_the_context_stays_usable(gpu):
    import torch
    lib, native = _lib()
    n = 1 << 22  # 512 tiles of 8192 keys per pass, 8 passes of the 63-bit key
    vert, faces = scenes.uniform_soup(n, seed=31)
    v = torch.from_numpy(vert).cuda()
    f = torch.from_numpy(faces.view(np.int32)).cuda()
    b = gpu.LBVH(n, 63, "karras")
    expected = b.build(v, f)
    torch.cuda.synchronize()
    assert b.errors() == 0
    prev = C.c_uint32()
    assert lib.bvhgb_sort_set_spin_limit(0, C.byref(prev)) == 0
    try:
        # the phases up to the sort only: its output is not a valid order after a timeout
        b.init_tri_data(v, f)
        b.calc_morton(v, f)
        b.sort(n)
        torch.cuda.synchronize()
        flags = b.errors()
    finally:
        assert lib.bvhgb_sort_set_spin_limit(0xFFFFFFFF, None) == 0
    assert prev.value == 1 << 24
    assert flags & TIMEOUT_BIT, flags
    # the context is intact and the next build is a normal one
    again = b.build(v, f)
    torch.cuda.synchronize()
    assert b.errors() == 0
    assert torch.equal(again, expected)
    b.close()


def _sweep(create, destroy, limit=64):
    """Fail the k-th allocation for k = 0, 1, ... until create succeeds; returns the number of
    allocations create makes. Every failing call must report OUT_OF_MEMORY."""
    lib, _ = _lib()
    try:
        for k in range(limit):
            assert lib.bvhgb_debug_fail_allocations(k, None) == 0
            st, handle = create()
            assert lib.bvhgb_debug_fail_allocations(-1, None) == 0
            if st == 0:
                destroy(handle)
                return k
            assert st == OUT_OF_MEMORY, (k, st)
    finally:
        lib.bvhgb_debug_fail_allocations(-1, None)
    raise AssertionError("create never succeeded")


def test_allocation_failures_give_out_of_memory_and_leak_nothing(gpu):
    import torch
    lib, native = _lib()
    n = 1 << 23
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()

    def lbvh():
        ws = C.c_void_p()
        cfg = native.LbvhConfig(63, 1)
        return lib.bvhgb_lbvh_create(n, C.byref(cfg), C.byref(ws)), ws

    counts = {"lbvh": _sweep(lbvh, lambda ws: lib.bvhgb_lbvh_destroy(ws))}

    m = 1 << 16
    vert, faces = scenes.uniform_soup(m, seed=32)
    v = torch.from_numpy(vert).cuda()
    f = torch.from_numpy(faces.view(np.int32)).cuda()
    nodes = gpu.LBVH(m, 30, "refCompat").build(v, f)
    torch.cuda.synchronize()

    def bn13():
        ws = C.c_void_p()
        cfg = native.Bn13Config(32, 128, 1.0, 0, 4096, 0, 0, 0)
        return lib.bvhgb_bn13_create(C.c_void_p(nodes.data_ptr()), 2 * m - 1, 0, C.byref(cfg), C.byref(ws), None), ws

    counts["bn13"] = _sweep(bn13, lambda ws: lib.bvhgb_bn13_destroy(ws))

    def tracer():
        tr = C.c_void_p()
        return lib.bvhgb_tracer_create(2 * n - 1, C.byref(tr)), tr

    counts["tracer"] = _sweep(tracer, lambda tr: lib.bvhgb_tracer_destroy(tr))

    def mesh():
        out = native.MeshRaw()
        return lib.bvhgb_copy_mesh_to_gpu(vert.ctypes.data_as(C.c_void_p), vert.shape[0], None, 0,
                                          faces.ctypes.data_as(C.c_void_p), faces.shape[0], C.byref(out)), out

    counts["mesh"] = _sweep(mesh, lambda out: lib.bvhgb_free_mesh(C.byref(out)))

    def bvh():
        out = native.BvhPointer()
        return lib.bvhgb_allocate_bvh(C.byref(out), n), out

    counts["bvh"] = _sweep(bvh, lambda out: lib.bvhgb_free_bvh(C.byref(out)))

    def mlp():
        h = C.c_void_p()
        return lib.bvhgb_mlp_create(7, C.byref(h)), h

    counts["mlp"] = _sweep(mlp, lambda h: lib.bvhgb_mlp_destroy(h))

    def features():
        h = C.c_void_p()
        return lib.bvhgb_lr_features_create(2 * n - 1, C.byref(h)), h

    counts["features"] = _sweep(features, lambda h: lib.bvhgb_lr_features_destroy(h))

    # every create allocates something, so every sweep saw at least one failure
    assert all(c >= 1 for c in counts.values()), counts
    del nodes, v, f
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free1, _ = torch.cuda.mem_get_info()
    # the LBVH workspace alone is about 0.4 GB, the tracer's records 0.5 GB: a leaked buffer of any
    # of the sweeps would show
    assert free0 - free1 < (32 << 20), (free0 - free1, counts)
