"""Writes tests/golden/oracle_small.npz: oracle outputs on small seeded scenes.

Run from the repository root:  python tests/golden/make_golden.py

The fixtures pin the oracle against later edits and give GPU tests a committed answer that does
not need the oracle at run time. The hand-derived values in known_answers.json come from the
reference's formulas worked on paper:
  * surface area of [0,1]x[0,2]x[0,3] = 2 (2 + 3 + 6) = 22 (lib/base/BVH.hpp:62-65);
  * inefficiency 2*4^3 / ((1 + 2) * 1) = 128/3, rounded to float (Bittner13CUDA.cu:493);
  * Morton codes with the scene box [0,1]^3 (offset 0, scale 1): 0.5 -> cell 512 -> bit 27, shifted
    by 2 / 1 / 0 for x / y / z (LBVH_CUDA.cu:132-166); 1.0 clamps to cell 1023 (all ones);
  * refCompat topology: the reference's delta is clz32(i ^ j) of the sorted positions, so the tree
    is the radix tree of 0..N-1 (N = 8: perfect; N = 5: root split 3 -> leaf 4 on the right);
  * karras topology of the 5-bit keys 00001 00010 00100 00101 10011 11000 11001 11110, the
    worked example of Karras (HPG 2012, fig. 4), numbered as kBuildTree does (LBVH_CUDA.cu:311-314);
  * adler32("Wikipedia") = 0x11E60398 (RFC 1950 definition).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from bvhtest_gb300 import scenes  # noqa: E402
from oracle import pyoracle as orc  # noqa: E402


def main():
    out = {}
    for n, seed in ((257, 11), (1000, 12)):
        vert, faces = scenes.uniform_soup(n, seed=seed)
        box, cen, scene = orc.tri_data(vert, faces)
        out[f"n{n}_vert"] = vert
        out[f"n{n}_scene"] = scene
        out[f"n{n}_morton30"] = orc.morton(cen, scene, 30)
        out[f"n{n}_morton63"] = orc.morton(cen, scene, 63)
        for bits in (30, 63):
            for mode, name in ((orc.REFCOMPAT, "ref"), (orc.KARRAS, "kar")):
                nodes, keys, idx = orc.lbvh_build(vert, faces, bits, mode)
                out[f"n{n}_b{bits}_{name}_nodes"] = nodes.view(np.uint8)
                out[f"n{n}_b{bits}_{name}_idx"] = idx
                out[f"n{n}_b{bits}_{name}_sah"] = np.float64(orc.sah(nodes))
    vert, faces = scenes.uniform_soup(1000, seed=12)
    nodes, _, _ = orc.lbvh_build(vert, faces, 30, orc.REFCOMPAT)
    org, dirs = orc.camera_rays((0.5, 0.5, -1.5), (0.5, 0.5, 0.0), (0, 1, 0), 60.0, 24, 16)
    hits = orc.trace_brute(org, dirs, vert, faces)
    out["img_dirs"] = dirs
    out["img_hits"] = hits.view(np.uint8)
    np.savez_compressed(Path(__file__).with_name("oracle_small.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
