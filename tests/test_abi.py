"""CPU checks of the C ABI: the library loads and exports every symbol include/*.h declares;
struct layouts match the reference's (lib/base/BVH.hpp). No compute calls (no GPU here)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names |= set(re.findall(r"BVHGB_API\s+[\w\s\*]+?\b(bvhgb_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    from bvhtest_gb300 import native
    lib = native.load()
    declared = _declared()
    assert len(declared) > 30
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(native.PROTOS) <= declared | {"bvhgb_trace_read_errors"}


def test_version_and_status_strings():
    from bvhtest_gb300 import native
    lib = native.load()
    assert b"sm_103a" in lib.bvhgb_version()
    assert lib.bvhgb_status_string(6) == b"CUDA_ERROR"
    assert lib.bvhgb_status_string(9) == b"DEVICE_TIMEOUT"


def test_argument_errors_without_gpu():
    """Invalid arguments are rejected on the host before any CUDA call."""
    from bvhtest_gb300 import native
    lib = native.load()
    assert lib.bvhgb_lbvh_create(10, None, None) == 8
    cfg = native.LbvhConfig(31, 0)
    ws = C.c_void_p()
    assert lib.bvhgb_lbvh_create(10, C.byref(cfg), C.byref(ws)) == 8
    cfg = native.LbvhConfig(30, 0)
    assert lib.bvhgb_lbvh_create(1 << 30, C.byref(cfg), C.byref(ws)) == 11
    need = C.c_size_t(0)
    assert lib.bvhgb_radix_sort_pairs(None, C.byref(need), None, None, None, None, 10, 3, 0, 8, None) == 8
    assert lib.bvhgb_select_smallest_pairs(None, C.byref(need), None, None, None, 10, 11, None) == 8  # k > n
    assert lib.bvhgb_select_smallest_pairs(None, None, None, None, None, 10, 5, None) == 8
    assert lib.bvhgb_trace_rays(None, 0, 0, None, None, None, None, 0, None, None, None) == 8
    assert lib.bvhgb_bn13_create(None, 0, 0, None, None, None) == 8


def test_struct_layouts():
    from bvhtest_gb300 import native
    assert native.NODE_DTYPE.itemsize == 48
    assert C.sizeof(native.Camera) == 48
    assert C.sizeof(native.MeshRaw) == 40
    assert C.sizeof(native.BvhPointer) == 24
    assert native.PIXEL_DTYPE.itemsize == 4


@pytest.mark.parametrize("field,off", [("parent", 24), ("left", 28), ("right", 32), ("isLeafFlag", 36),
                                       ("isLeft", 38), ("level", 40), ("surfaceArea", 44)])
def test_node_offsets(field, off):
    from bvhtest_gb300 import native
    assert native.NODE_DTYPE.fields[field][1] == off


def test_every_entry_rejects_null_handles_without_crashing():
    """Every exported function called with null pointers and zero sizes returns a status: invalid
    argument for a missing handle or buffer, OK where null is allowed (destroy, queries), a CUDA
    error where the device itself is needed. Nothing dereferences the null."""
    from bvhtest_gb300 import native
    lib = native.load()
    allowed_ok = {"bvhgb_sort_set_default_tile"}  # tileKeys = 0 with a null 'previous' only reads
    # process-wide diagnostic settings, not handle functions: zeros would change later calls
    settings = {"bvhgb_sort_set_spin_limit", "bvhgb_debug_fail_allocations"}
    for name in sorted(set(native.PROTOS) - settings):
        f = getattr(lib, name)
        args = []
        for t in f.argtypes or []:
            if t in (C.c_float, C.c_double):
                args.append(0.0)
            elif t in (C.c_void_p, C.c_char_p) or (isinstance(t, type) and issubclass(t, C._Pointer)):
                args.append(None)
            else:
                args.append(0)
        r = f(*args)
        if f.restype is not C.c_int32 or not f.argtypes:
            continue  # counters, strings, sizes; bvhgb_device_sync needs a device
        if name.endswith("_destroy") or name in allowed_ok:
            assert r == 0, name
        else:
            assert r == 8, (name, r)  # BVHGB_INVALID_ARGUMENT


def test_allocation_free_build_argument_checks_without_gpu():
    """bvhgb_lbvh_build_static and its error read-back reject bad arguments on the host, before any
    device call: nothing to build (numFaces = 0) is OK, missing buffers and bad configurations are
    invalid arguments, sizes above the array's maximum are too large."""
    from bvhtest_gb300 import native
    lib = native.load()
    build = lib.bvhgb_lbvh_build_static
    build.restype = C.c_int
    build.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.POINTER(native.LbvhConfig), C.c_void_p, C.c_void_p]
    read = lib.bvhgb_lbvh_static_read_errors
    read.restype = C.c_int
    read.argtypes = [C.POINTER(native.LbvhConfig), C.POINTER(C.c_uint32), C.c_void_p]
    assert build(None, None, 0, None, None, None) == 0
    assert build(None, None, 10, None, None, None) == 8
    bad = native.LbvhConfig(31, 0)
    assert build(None, None, 10, C.byref(bad), None, None) == 8
    assert build(None, None, 262144 + 1, None, None, None) == 11
    flags = C.c_uint32()
    assert read(None, None, None) == 8
    assert read(C.byref(bad), C.byref(flags), None) == 8
