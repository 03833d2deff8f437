"""In-tree build of the CUDA library (sm_103a) and the native host layer.

Every translation unit is compiled in parallel with nvcc / g++ and linked into
bvhtest_gb300/lib/libbvhgb.so and the bvhTest command-line runner. Nothing is installed outside
the source tree.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
OBJ = PKG / "_build"
LIB = PKG / "lib"
LIBNAME = "libbvhgb.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
    "-I" + str(ROOT / "include"),
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fvisibility=hidden",
             "-I" + str(ROOT / "include"), "-Wall", "-Wno-unused-function"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA library cannot be built")


def _cuda_lib_dir() -> str:
    nvcc = Path(_nvcc()).resolve()
    root = nvcc.parent.parent
    for cand in (root / "lib64", root / "targets" / "sbsa-linux" / "lib", root / "targets" / "x86_64-linux" / "lib"):
        if (cand / "libcudart.so").exists() or (cand / "libcudart_static.a").exists():
            return str(cand)
    return str(root / "lib64")


def _cuda_include_dir() -> str:
    root = Path(_nvcc()).resolve().parent.parent
    for cand in (root / "include", root / "targets" / "sbsa-linux" / "include",
                 root / "targets" / "x86_64-linux" / "include"):
        if (cand / "cuda_runtime.h").exists():
            return str(cand)
    return str(root / "include")


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(HOST.glob("*.cpp")) if HOST.exists() else []
    return cu, cpp


def _stamp(paths, flags) -> str:
    h = hashlib.sha256()
    for p in sorted(paths):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(cmd), res.stdout, res.stderr))
    return res


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile and link libbvhgb.so (and the bvhTest runner). Returns the library path."""
    cu, cpp = _sources()
    headers = list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")) + list(HOST.glob("*.hpp"))
    nvcc = _nvcc()
    stamp = _stamp(cu + cpp + headers, ARCH + NVCC_FLAGS + CXX_FLAGS + [os.uname().machine])
    LIB.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    lib = LIB / LIBNAME
    stamp_file = OBJ / "stamp"
    if not force and lib.exists() and stamp_file.exists() and stamp_file.read_text() == stamp:
        return lib
    jobs = []
    for src in cu:
        jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(OBJ / (src.stem + ".o"))])
    host_lib_objs = []
    for src in cpp:
        if src.name == "main.cpp":
            continue
        out = OBJ / ("host_" + src.stem + ".o")
        host_lib_objs.append(out)
        jobs.append(["g++", *CXX_FLAGS, "-I" + _cuda_include_dir(), "-c", str(src), "-o", str(out)])
    with ThreadPoolExecutor(max_workers=max(2, min(len(jobs), os.cpu_count() or 4))) as ex:
        for res in ex.map(_run, jobs):
            if verbose and (res.stdout or res.stderr):
                print(res.stdout, res.stderr)
    objs = [str(OBJ / (s.stem + ".o")) for s in cu] + [str(o) for o in host_lib_objs]
    tmp = lib.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-o", str(tmp), *objs, "-Xlinker", "-rpath,$ORIGIN", "-lcudart"])
    os.replace(tmp, lib)
    main = HOST / "main.cpp"
    if main.exists():
        exe = LIB / "bvhTest"
        _run(["g++", *CXX_FLAGS, str(main), "-o", str(exe), "-L" + str(LIB), "-lbvhgb",
              "-Wl,-rpath,$ORIGIN", "-L" + _cuda_lib_dir(), "-lcudart"])
    stamp_file.write_text(stamp)
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force=True))
