"""Build recipe for the CPU oracle (test infrastructure only): gcc -> oracle/_build/liborc.so.

-ffp-contract=off keeps every a*b+c as two rounded operations on both x86-64 and aarch64, which
is the convention the GPU kernels follow with explicit __fmul_rn/__fadd_rn.
"""
from __future__ import annotations

import hashlib
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
SOURCES = ["lbvh.c", "bittner.c", "tracer.c", "learned.c"]
CXX_SOURCES = ["stdselect.cpp"]  # the reference optimizers' std::nth_element / std::sort order
FLAGS = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
         "-Wall", "-Wno-unused-function"]


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    lib = OUT / "liborc.so"
    h = hashlib.sha256()
    for s in SOURCES + CXX_SOURCES + ["oracle.h"]:
        h.update((HERE / s).read_bytes())
    h.update(" ".join(FLAGS).encode())
    stamp = OUT / "stamp"
    if not force and lib.exists() and stamp.exists() and stamp.read_text() == h.hexdigest():
        return lib
    obj = OUT / "stdselect.o"
    cxx = ["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-Wall",
           "-c", str(HERE / CXX_SOURCES[0]), "-o", str(obj)]
    cmd = ["gcc", *FLAGS, *[str(HERE / s) for s in SOURCES], str(obj), "-o", str(lib) + ".tmp", "-lm", "-lstdc++"]
    for c in (cxx, cmd):
        res = subprocess.run(c, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + res.stdout + res.stderr)
    Path(str(lib) + ".tmp").replace(lib)
    stamp.write_text(h.hexdigest())
    return lib


if __name__ == "__main__":
    print(build(force=True))
