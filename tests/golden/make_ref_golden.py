"""Writes tests/golden/ref_pin.npz: outputs of the reference's OWN CPU code (oracle/_ref, compiled
from the reference's sources by oracle/build_ref.py) on the seeded scenes of the workloads, so that
machines without the reference (the GPU machine) still check against it.

Run from the repository root, where the reference's sources are present:
    python tests/golden/make_ref_golden.py [--parts c1,c2,c5]

Contents (all trees start from the oracle's LBVH, which equals the GPU's bit for bit):
  c1_*  uniform 65,536 triangles (seed 1), 30-bit refCompat LBVH:
        Bittner13 (sequential) and Bittner13Par (32 chunks, 1 thread) for 100 iterations at 1%:
        the reference's own float SAH after every iteration, the SHA-256 of the final node array
        (levels fixed by the reference's teardown), Bittner13Par's skip count; Bittner13Par with
        altFindNode (16 queue slots) for 20 iterations: tree hash and skip count;
        the camera's 512 x 512 primary rays (SHA-256 of directions) and the CPUTracer image
        (SHA-256 of the grey values, the inner-node visit counts and the hit mask).
  c2_*  large scene (4,194,304 triangles, seed 2), 63-bit karras LBVH: Bittner13 and Bittner13Par
        (32 chunks, all host threads) for 200 iterations at 1%, the SAH (summed in double by the
        oracle) of the reference's tree after every iteration.
  c5_*  stress scene (33,554,432 triangles, seed 5), 63-bit karras LBVH: both optimizers for
        C5_ITERS iterations, SAH after every iteration as above.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from bvhtest_gb300 import scenes  # noqa: E402
from oracle import pyoracle as orc  # noqa: E402
from oracle import refpy  # noqa: E402

OUT = Path(__file__).with_name("ref_pin.npz")
C1_ITERS = 100
C1_ALT_ITERS = 20  # Bittner13Par with altFindNode (the 16-slot queue of findNode2)
C2_ITERS = 200
C5_ITERS = 20
THREADS = os.cpu_count() or 1


def sha(a) -> np.ndarray:
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), np.uint8)


def stepwise(fn, nodes, iters):
    """Runs a reference optimizer one iteration per call (each call re-reads the tree, so this equals
    one call of `iters` iterations) and takes the oracle's double SAH after every iteration."""
    trace = [orc.sah(nodes)]
    for _ in range(iters):
        nodes = fn(nodes)
        trace.append(orc.sah(nodes))
    return nodes, np.array(trace, np.float64)


def part_c1(out):
    vert, faces = scenes.uniform_soup(65536, seed=1)
    nodes, _, _ = orc.lbvh_build(vert, faces, 30, orc.REFCOMPAT)
    a, sa, st = refpy.bittner13(nodes, C1_ITERS, threads=1)
    assert st == 0
    out["c1_seq_sah"] = sa
    out["c1_seq_sha"] = sha(a)
    b, sb, sk, tot, st = refpy.bittner13par(nodes, C1_ITERS, threads=1)
    assert st == 0
    out["c1_par_sah"] = sb
    out["c1_par_sha"] = sha(b)
    out["c1_par_skipped"] = np.uint32(sk)
    out["c1_par_total"] = np.uint32(tot)
    c, _, sk, _, st = refpy.bittner13par(nodes, C1_ALT_ITERS, alt_find_node=True, alt_queue=16, threads=1)
    assert st == 0
    out["c1_par_alt_sha"] = sha(c)
    out["c1_par_alt_skipped"] = np.uint32(sk)
    cam = scenes.camera_default()
    c = (cam["pos"], cam["lookAt"], cam["up"], cam["fov"], cam["width"], cam["height"])
    _, dirs = refpy.camera_rays(*c)
    out["c1_rays_sha"] = sha(dirs)
    grey, cnt, hit, _ = refpy.trace(nodes, vert, faces, c)
    out["c1_trace_grey_sha"] = sha(grey)
    out["c1_trace_count_sha"] = sha(cnt)
    out["c1_trace_hit_sha"] = sha(hit.astype(np.uint8))
    out["c1_trace_hits"] = np.uint32(hit.sum())


def part_large(out, key, vert, faces, iters):
    nodes, _, _ = orc.lbvh_build(vert, faces, 63, orc.KARRAS)
    del vert, faces
    out[f"{key}_start_sah"] = np.float64(orc.sah(nodes))
    t = time.time()
    _, tr = stepwise(lambda x: refpy.bittner13(x, 1, threads=THREADS)[0], nodes, iters)
    out[f"{key}_seq_sah"] = tr
    print(key, "Bittner13", iters, "iterations", round(time.time() - t, 1), "s, SAH", tr[-1], flush=True)
    t = time.time()
    _, tr = stepwise(lambda x: refpy.bittner13par(x, 1, threads=THREADS)[0], nodes, iters)
    out[f"{key}_par_sah"] = tr
    print(key, "Bittner13Par", iters, "iterations", round(time.time() - t, 1), "s, SAH", tr[-1], flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--parts", default="c1,c2,c5")
    args = ap.parse_args()
    if refpy.lib() is None:
        raise SystemExit("the reference's sources are needed (oracle/build_ref.py)")
    out = dict(np.load(OUT)) if OUT.exists() else {}
    parts = args.parts.split(",")
    if "c1" in parts:
        part_c1(out)
    if "c2" in parts:
        vert, faces = scenes.large_scene()
        part_large(out, "c2", vert, faces, C2_ITERS)
    if "c5" in parts:
        vert, faces = scenes.stress_scene()
        part_large(out, "c5", vert, faces, C5_ITERS)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, len(out), "arrays")


if __name__ == "__main__":
    main()
