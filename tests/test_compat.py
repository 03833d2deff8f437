"""The reference's own GPU entry points (include/bvhtest_compat.h) exported by libbvhgb.so.

* Link check (CPU, where the reference's sources are present): the reference's command files
  lib/builder/LBVH.cpp, Bittner13GPU.cpp, lib/tracer/CUDATracer.cpp, lib/cuda/CopyToGPU.cpp and
  CopyToHost.cpp, compiled unchanged from the reference's tree, link against libbvhgb.so with no
  undefined symbol: the library is a relink-level drop-in for LBVH_CUDA.cu, Bittner13CUDA.cu,
  CUDAKernels.cu and cudaFN.cu.
* Pipeline (GPU): tests/compat_driver.cpp calls only those entry points, in the command files'
  order, and its LBVH tree, optimised tree, SAH trace and traced image equal the oracle's.
"""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from bvhtest_gb300 import scenes

ROOT = Path(__file__).resolve().parent.parent
LIB = ROOT / "bvhtest_gb300" / "lib"
REF_COMMANDS = ["lib/builder/LBVH.cpp", "lib/builder/Bittner13GPU.cpp", "lib/tracer/CUDATracer.cpp",
                "lib/cuda/CopyToGPU.cpp", "lib/cuda/CopyToHost.cpp"]
COMPAT_SYMBOLS = ["LBVH_initTriData", "LBVH_calcMortonCodes", "LBVH_sortMortonCodes", "LBVH_buildBVHTree",
                  "LBVH_fixAABB", "LBVH_allocateBVH", "LBVH_allocateWorkingMemory", "LBVH_freeWorkingMemory",
                  "LBVH_doCUDASyc", "allocateMemory", "freeMemory", "initData", "fixTree1", "fixTree3",
                  "bn13_selectNodes", "bn13_rmAndReinsChunk", "bn13_doAlgorithmStep", "CUDAcalcSAH",
                  "doCudaDevSync", "calcNumSkipped", "allocateRays", "allocateImage", "freeRays", "freeImage",
                  "generateRays", "tracerImage", "copyImageToHost", "tracerDoCudaSync", "copyBVHToGPU",
                  "copyMeshToGPU", "copyBVHToHost", "copyMeshToHost", "resetCUDA"]


def _cuda_lib_dir():
    from bvhtest_gb300 import _build
    return _build._cuda_lib_dir()


def _lib():
    from bvhtest_gb300 import _build
    return _build.build()


def test_library_exports_every_reference_entry_point():
    lib = _lib()
    out = subprocess.run(["nm", "-DC", "--defined-only", str(lib)], capture_output=True, text=True, check=True).stdout
    names = set()
    for line in out.splitlines():
        parts = line.split(" ", 2)
        if len(parts) == 3:
            names.add(parts[2].split("(")[0])
    missing = [s for s in COMPAT_SYMBOLS if s not in names]
    assert not missing, missing


def _build_driver(tmp_path):
    exe = tmp_path / "compat_driver"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + str(ROOT / "include"), str(ROOT / "tests" / "compat_driver.cpp"),
                    "-o", str(exe), "-L" + str(LIB), "-lbvhgb", "-Wl,-rpath," + str(LIB), "-L" + _cuda_lib_dir(),
                    "-lcudart", "-Wl,--no-undefined"], check=True, capture_output=True, text=True)
    return exe


def test_compat_driver_builds_against_the_header(tmp_path):
    _lib()
    assert _build_driver(tmp_path).exists()


def test_reference_command_files_link_against_the_library(tmp_path):
    from oracle import build_ref, refpy
    if refpy.lib() is None:
        pytest.skip("the reference's sources are not on this machine")
    lib = _lib()
    ref = build_ref.REF
    inc = ["-I" + str(ROOT / "oracle" / "refshim"), "-I" + str(ref / "lib"), "-I" + str(ref / "external")]
    objs = []
    for src in REF_COMMANDS:
        o = tmp_path / (Path(src).stem + ".o")
        subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-w", *inc, "-c", str(ref / src), "-o", str(o)],
                       check=True, capture_output=True, text=True)
        objs.append(str(o))
    main = tmp_path / "main.cpp"
    main.write_text(
        '#include "builder/LBVH.hpp"\n#include "builder/Bittner13GPU.hpp"\n#include "tracer/CUDATracer.hpp"\n'
        '#include "cuda/CopyToGPU.hpp"\n#include "cuda/CopyToHost.hpp"\n'
        "int main() {\n  BVHTest::builder::LBVH a; BVHTest::builder::Bittner13GPU b; BVHTest::tracer::CUDATracer c;\n"
        "  BVHTest::cuda::CopyToGPU d; BVHTest::cuda::CopyToHost e;\n"
        "  return a.getName().empty() + b.getName().empty() + c.getName().empty() + d.getName().empty()"
        " + e.getName().empty();\n}\n")
    subprocess.run(["g++", "-std=c++17", "-O1", "-w", *inc, "-c", str(main), "-o", str(tmp_path / "main.o")],
                   check=True, capture_output=True, text=True)
    # the reference's base classes (Command, Configurable, OptimizerBase, TracerBase ...) come from
    # the objects oracle/build_ref.py compiled from the same tree
    base = [str(build_ref.OUT / (n + ".o")) for n in ("BVH", "Ray", "Configurable", "CameraBase", "OptimizerBase",
                                                      "BuilderBase", "TracerBase", "Camera", "ref_harness",
                                                      "Bittner13", "Bittner13Par", "Wald07", "Median", "CPUTracer",
                                                      "BruteForceTracer")]
    res = subprocess.run(["g++", "-o", str(tmp_path / "commands"), str(tmp_path / "main.o"), *objs, *base,
                          "-L" + str(lib.parent), "-lbvhgb", "-L" + _cuda_lib_dir(), "-lcudart", "-fopenmp",
                          "-Wl,--no-undefined"], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]
    # and every bvh symbol those files need is undefined in them, i.e. provided by libbvhgb.so
    und = subprocess.run(["nm", "-uC", *objs], capture_output=True, text=True, check=True).stdout
    needed = {s for s in COMPAT_SYMBOLS if s in und}
    assert {"LBVH_initTriData", "bn13_doAlgorithmStep", "tracerImage", "copyBVHToHost", "resetCUDA"} <= needed


@pytest.mark.gpu
def test_pipeline_through_the_reference_entry_points(orc, tmp_path):
    exe = _build_driver(tmp_path)
    n, iters, w, h = 16384, 10, 256, 256
    vert, faces = scenes.uniform_soup(n, seed=17)
    ind, outd = tmp_path / "in", tmp_path / "out"
    ind.mkdir()
    outd.mkdir()
    vert.astype(np.float32).tofile(ind / "vert.bin")
    faces.astype(np.uint32).tofile(ind / "faces.bin")
    res = subprocess.run([str(exe), str(ind), str(outd), str(iters), str(w), str(h)], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    lbvh = np.fromfile(outd / "lbvh.bin", orc.NODE_DTYPE)
    ref, _, _ = orc.lbvh_build(vert, faces, 30, orc.REFCOMPAT)
    assert np.array_equal(lbvh.view(np.uint8), ref.view(np.uint8))
    opt = np.fromfile(outd / "opt.bin", orc.NODE_DTYPE)
    ropt, trace, st = orc.bittner_chunked(ref, iters)
    assert np.array_equal(opt.view(np.uint8), ropt.view(np.uint8))
    sah = np.fromfile(outd / "sah.bin", np.float32)
    assert np.allclose(sah, trace.astype(np.float32), rtol=1e-6, atol=0)
    skipped, total = map(int, (outd / "skipped.txt").read_text().split())
    assert skipped == st["skipped_conflict"] + st["skipped_invalid"] and total == st["items"]
    # the reference's tracer culls back faces by default (CUDA_FACE_CULLING)
    px = np.fromfile(outd / "img.bin", np.dtype([("hit", "u1"), ("diffuse", "u1"), ("intCount", "<u2")]))
    org, dirs = orc.camera_rays((0.5, 0.5, -1.5), (0.5, 0.5, 0.0), (0, 1, 0), 60.0, w, h)
    hits = orc.trace_bvh(org, dirs, ropt, vert, faces, cull=True)
    hit = hits["prim"] != 0xFFFFFFFF
    assert hit.mean() > 0.02
    assert np.array_equal(px["hit"], hit.astype(np.uint8))
    for i in np.nonzero(hit)[0][::41]:
        tri = faces[hits["prim"][i]]
        assert px["diffuse"][i] == orc.shade(org[i], dirs[i], hits["t"][i], vert[tri[0]], vert[tri[1]], vert[tri[2]])
    # rayBundles: the same pixels; intCount counts the bundle's visits, at least each ray's own
    bundle = np.fromfile(outd / "img_bundle.bin", px.dtype)
    assert np.array_equal(bundle["hit"], px["hit"]) and np.array_equal(bundle["diffuse"], px["diffuse"])
    assert (bundle["intCount"] >= px["intCount"]).all()
    assert np.array_equal(np.fromfile(outd / "mesh_vert.bin", np.float32), vert.astype(np.float32).ravel())
