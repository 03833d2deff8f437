"""Build recipe for oracle/_ref/libref.so (test infrastructure only): the reference's own CPU
sources, compiled where they lie, plus oracle/ref_harness.cpp, which exposes their command classes
through plain C entry points.

The reference's math, formatting and logging submodules are empty in its tree, and its config
header is generated by its build system; oracle/refshim/ holds this project's stand-ins for them
(written from the published definitions; see the header comments there). The reference's
nlohmann json header is taken from its external/ folder. The reference's build system is not
used: g++ compiles the listed files directly.

Only this container has the reference; on a machine without it, build() returns None and the
tests that need the library skip (the committed fixtures under tests/golden/ carry its outputs).
CPUTracer.cpp and BruteForceTracer.cpp time rays with the x86 time-stamp counter, so the library
builds on x86-64 only.
"""
from __future__ import annotations

import hashlib
import os
import platform
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
REF = Path(os.environ.get("BVHTEST_REFERENCE", "/root/reference"))

# Every reference file the pinned paths need (file paths inside the reference project).
REF_SOURCES = [
    "lib/base/BVH.cpp",
    "lib/base/Ray.cpp",
    "lib/base/Configurable.cpp",
    "lib/base/CameraBase.cpp",
    "lib/builder/OptimizerBase.cpp",
    "lib/builder/Bittner13.cpp",
    "lib/builder/Bittner13Par.cpp",
    "lib/builder/BuilderBase.cpp",
    "lib/builder/Wald07.cpp",
    "lib/builder/Median.cpp",
    "lib/misc/Camera.cpp",
    "lib/tracer/TracerBase.cpp",
    "lib/tracer/CPUTracer.cpp",
    "lib/tracer/BruteForceTracer.cpp",
]
FLAGS = ["-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-w"]


def available() -> bool:
    return (REF / "lib" / "builder" / "Bittner13.cpp").exists() and platform.machine() in ("x86_64", "AMD64")


def _includes():
    return ["-I" + str(HERE / "refshim"), "-I" + str(REF / "lib"), "-I" + str(REF / "external")]


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference build failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))


def build(force: bool = False):
    """Compile the reference's CPU sources into oracle/_ref/libref.so; None without the reference."""
    if not available():
        return None
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libref.so"
    srcs = [REF / s for s in REF_SOURCES] + [HERE / "ref_harness.cpp"]
    h = hashlib.sha256()
    for p in srcs + sorted((HERE / "refshim").rglob("*")):
        if p.is_file():
            h.update(str(p).encode())
            h.update(p.read_bytes())
    h.update(" ".join(FLAGS).encode())
    stamp = OUT / "stamp"
    if not force and lib.exists() and stamp.exists() and stamp.read_text() == h.hexdigest():
        return lib
    objs = []
    jobs = []
    for s in srcs:
        o = OUT / (s.stem + ".o")
        objs.append(str(o))
        jobs.append(["g++", *FLAGS, *_includes(), "-c", str(s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 4)) as ex:
        list(ex.map(_run, jobs))
    _run(["g++", "-shared", "-fopenmp", "-o", str(lib) + ".tmp", *objs])
    Path(str(lib) + ".tmp").replace(lib)
    stamp.write_text(h.hexdigest())
    return lib


if __name__ == "__main__":
    print(build(force=True))
