"""CPU tests of the oracle: hand-derived known answers, committed fixtures, invariants.

The reference ships no tests or golden vectors, so these pin the oracle to the reference's
formulas worked by hand (tests/golden/known_answers.json) and to its runtime invariants
(lib/misc/Validate.cpp restated in oracle/lbvh.c).
"""
import json
import struct
from pathlib import Path

import numpy as np
import pytest

from bvhtest_gb300 import scenes

GOLDEN = Path(__file__).resolve().parent / "golden"
KA = json.loads((GOLDEN / "known_answers.json").read_text())


def test_node_layout(orc):
    assert orc.NODE_DTYPE.itemsize == 48
    assert orc.NODE_DTYPE.fields["parent"][1] == 24
    assert orc.NODE_DTYPE.fields["isLeafFlag"][1] == 36
    assert orc.NODE_DTYPE.fields["surfaceArea"][1] == 44


def test_surface_area_and_cost(orc):
    import ctypes as C
    b = orc.Aabb((C.c_float * 3)(0, 0, 0), (C.c_float * 3)(1, 2, 3))
    assert orc.lib().orc_surface_area(C.byref(b)) == KA["surface_area"]["sa"]
    nodes = np.zeros(3, orc.NODE_DTYPE)
    nodes[0]["left"], nodes[0]["right"] = 1, 2
    nodes[0]["surfaceArea"], nodes[1]["surfaceArea"], nodes[2]["surfaceArea"] = 4.0, 1.0, 2.0
    nodes[1]["isLeafFlag"] = nodes[2]["isLeafFlag"] = 1
    c = orc.lib().orc_inefficiency(nodes.ctypes.data_as(C.c_void_p), 0)
    assert struct.unpack("<I", struct.pack("<f", c))[0] == int(KA["inefficiency"]["cost_f32_bits"], 16)
    assert orc.lib().orc_inefficiency(nodes.ctypes.data_as(C.c_void_p), 1) == 0.0


def test_morton_known_answers(orc):
    k = KA["morton30"]
    codes = orc.morton(np.array(k["centroids"], np.float32), np.array(k["scene"], np.float32), 30)
    assert codes.tolist() == k["codes"]
    c63 = orc.morton(np.array([[1, 1, 1], [0.5, 0, 0]], np.float32), np.array(k["scene"], np.float32), 63)
    assert int(c63[0]) == (1 << 63) - 1
    assert int(c63[1]) == 1 << 62


def test_scene_box_includes_origin(orc):
    # LBVH_CUDA.cu:104-106: the reduction starts from the box [(0,0,0),(0,0,0)].
    vert = np.array([[2, 3, 4], [3, 3, 4], [2, 4, 5]], np.float32)
    faces = np.array([[0, 1, 2]], np.uint32)
    _, cen, scene = orc.tri_data(vert, faces)
    assert scene[:3].tolist() == [0.0, 0.0, 0.0]
    eps = np.float32(np.finfo(np.float32).eps)
    assert scene[3:].tolist() == [np.float32(3) + eps, np.float32(4) + eps, np.float32(5) + eps]
    assert np.allclose(cen[0], [7 / 3, 10 / 3, 13 / 3])


@pytest.mark.parametrize("n", ["5", "8"])
def test_refcompat_topology_known_answer(orc, n):
    import ctypes as C
    n_i = int(n)
    nodes = np.zeros(2 * n_i - 1, orc.NODE_DTYPE)
    keys = np.arange(n_i, dtype=np.uint32)[::-1].copy()  # codes are ignored by refCompat
    orc.lib().orc_build_topology(keys.ctypes.data_as(C.c_void_p), None, n_i, 0, nodes.ctypes.data_as(C.c_void_p))
    exp = KA["refcompat_topology"][n]
    assert nodes["left"][: n_i - 1].tolist() == exp["left"]
    assert nodes["right"][: n_i - 1].tolist() == exp["right"]


def test_karras_topology_known_answer(orc):
    import ctypes as C
    k = KA["karras_topology"]
    keys = np.array(k["keys"], np.uint32)
    nodes = np.zeros(2 * len(keys) - 1, orc.NODE_DTYPE)
    orc.lib().orc_build_topology(keys.ctypes.data_as(C.c_void_p), None, len(keys), 1, nodes.ctypes.data_as(C.c_void_p))
    assert nodes["left"][: len(keys) - 1].tolist() == k["left"]
    assert nodes["right"][: len(keys) - 1].tolist() == k["right"]
    # 64-bit keys holding the same codes give the same tree.
    k64 = keys.astype(np.uint64)
    n2 = np.zeros_like(nodes)
    orc.lib().orc_build_topology(None, k64.ctypes.data_as(C.c_void_p), len(keys), 1, n2.ctypes.data_as(C.c_void_p))
    assert n2["left"][: len(keys) - 1].tolist() == k["left"]


def test_sort_is_stable(orc):
    g = np.random.default_rng(5)
    keys = g.integers(0, 50, 10000).astype(np.uint32)
    ko, vo = orc.sort_pairs(keys)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(vo, order) and np.array_equal(ko, keys[order])
    k64 = g.integers(0, 1 << 62, 5000, dtype=np.uint64)
    ko, vo = orc.sort_pairs(k64)
    assert np.array_equal(vo, np.argsort(k64, kind="stable"))


@pytest.mark.parametrize("n", [1, 2, 3, 5, 1000, 4097])
@pytest.mark.parametrize("bits,mode", [(30, 0), (30, 1), (63, 1), (63, 0)])
def test_lbvh_valid(orc, n, bits, mode):
    vert, faces = scenes.uniform_soup(n, seed=n)
    nodes, keys, idx = orc.lbvh_build(vert, faces, bits, mode)
    assert nodes.shape[0] == 2 * n - 1
    assert orc.validate(nodes, vert, faces) == [0, 0, 0, 0, 0]
    assert np.all(np.diff(keys.astype(np.uint64).astype(object) if bits == 63 else keys.astype(np.int64)) >= 0)
    assert sorted(idx.tolist()) == list(range(n))
    assert nodes[0]["parent"] == 0
    if n > 1:
        assert np.all(nodes["isLeafFlag"][: n - 1] == 0) and np.all(nodes["isLeafFlag"][n - 1:] == 1)
        assert np.all(nodes["level"][n - 1:] == 255)


def test_lbvh_matches_committed_fixtures(orc):
    g = np.load(GOLDEN / "oracle_small.npz")
    for n, seed in ((257, 11), (1000, 12)):
        vert, faces = scenes.uniform_soup(n, seed=seed)
        assert np.array_equal(vert, g[f"n{n}_vert"])
        for bits in (30, 63):
            for mode, name in ((0, "ref"), (1, "kar")):
                nodes, _, idx = orc.lbvh_build(vert, faces, bits, mode)
                assert np.array_equal(nodes.view(np.uint8), g[f"n{n}_b{bits}_{name}_nodes"])
                assert np.array_equal(idx, g[f"n{n}_b{bits}_{name}_idx"])


def test_karras_mode_has_lower_sah(orc):
    vert, faces = scenes.uniform_soup(20000, seed=3)
    ref, _, _ = orc.lbvh_build(vert, faces, 30, 0)
    kar, _, _ = orc.lbvh_build(vert, faces, 30, 1)
    assert orc.sah(kar) < orc.sah(ref)


def test_validate_catches_planted_errors(orc):
    vert, faces = scenes.uniform_soup(100, seed=4)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    bad = nodes.copy()
    bad[5]["parent"] = 7
    assert orc.validate(bad, vert, faces)[0] > 0
    bad = nodes.copy()
    bad[3]["mn"][0] += 0.5
    e = orc.validate(bad, vert, faces)
    assert e[1] > 0 or e[2] > 0 or e[3] > 0
    bad = nodes.copy()
    bad[150]["surfaceArea"] += 1e-3
    assert orc.validate(bad, vert, faces)[3] > 0


def test_fix_levels(orc):
    vert, faces = scenes.uniform_soup(64, seed=5)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    assert orc.fix_levels(nodes) == 6  # refCompat over 64 keys is a perfect tree
    assert orc.validate(nodes, vert, faces, check_levels=True) == [0, 0, 0, 0, 0]


def test_watertight_known_answer(orc):
    w = KA["watertight"]
    hit, t = orc.ray_tri(w["org"], w["dir"], *w["tri"])
    assert hit and t == w["t"]
    hit_c, _ = orc.ray_tri(w["org"], w["dir"], *w["tri"], cull=True)
    assert hit_c is (not w["back_facing"])
    # Flipping the winding makes it front facing.
    hit_f, t_f = orc.ray_tri(w["org"], w["dir"], w["tri"][0], w["tri"][2], w["tri"][1], cull=True)
    assert hit_f and t_f == w["t"]


def test_watertight_shared_edge(orc):
    # Rays through the shared edge of two triangles hit exactly one or both, never neither.
    quad = [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]]
    g = np.random.default_rng(6)
    for _ in range(500):
        s = g.random()
        org = [s, s, -1.0]  # lies over the diagonal (0,0)-(1,1)
        d = [0.0, 0.0, 1.0]
        a, _ = orc.ray_tri(org, d, quad[0], quad[1], quad[2])
        b, _ = orc.ray_tri(org, d, quad[0], quad[2], quad[3])
        assert a or b


def test_camera_center_ray(orc):
    c = KA["camera_center"]
    org, dirs = orc.camera_rays(c["pos"], c["lookAt"], c["up"], c["fov"], c["width"], c["height"])
    assert dirs[0].tolist() == c["dir"]
    assert org[0].tolist() == [np.float32(x) for x in c["pos"]]


def test_bvh_trace_equals_brute_force(orc):
    vert, faces = scenes.uniform_soup(3000, seed=7)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    org, dirs = orc.camera_rays((0.5, 0.5, -1.5), (0.5, 0.5, 0.0), (0, 1, 0), 60.0, 64, 64)
    hb = orc.trace_brute(org, dirs, vert, faces)
    hv = orc.trace_bvh(org, dirs, nodes, vert, faces)
    assert np.array_equal(hb["prim"], hv["prim"]) and np.array_equal(hb["t"], hv["t"])
    assert (hb["prim"] != 0xFFFFFFFF).sum() > 20  # ~1% of the view is covered by 3000 tiny triangles
    ro, rd = scenes.random_rays(4000, (-0.5, -0.5, -0.5), (1.5, 1.5, 1.5), seed=8)
    hb = orc.trace_brute(ro, rd, vert, faces)
    hv = orc.trace_bvh(ro, rd, nodes, vert, faces)
    assert np.array_equal(hb["prim"], hv["prim"])


def test_golden_image_hits(orc):
    g = np.load(GOLDEN / "oracle_small.npz")
    vert, faces = scenes.uniform_soup(1000, seed=12)
    org, dirs = orc.camera_rays((0.5, 0.5, -1.5), (0.5, 0.5, 0.0), (0, 1, 0), 60.0, 24, 16)
    assert np.array_equal(dirs, g["img_dirs"])
    assert np.array_equal(orc.trace_brute(org, dirs, vert, faces).view(np.uint8), g["img_hits"])


def test_cpu_reference_tracer_agrees_mostly(orc):
    # The reference CPU tracer (two-sided double Moller-Trumbore) and the watertight oracle agree
    # on nearly every pixel of a triangle soup; they may differ only at edges.
    vert, faces = scenes.uniform_soup(3000, seed=7)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    org, dirs = orc.camera_rays((0.5, 0.5, -1.5), (0.5, 0.5, 0.0), (0, 1, 0), 60.0, 64, 64)
    hb = orc.trace_brute(org, dirs, vert, faces)
    hr, cnt = orc.trace_cpu_reference(org, dirs, nodes, vert, faces)
    assert (hb["prim"] == hr["prim"]).mean() > 0.995
    assert cnt.max() > 0


def test_adler32(orc):
    assert orc.adler32(KA["adler32"]["text"].encode()) == int(KA["adler32"]["value"], 16)


def test_bittner_sequential_improves_and_stays_valid(orc):
    vert, faces = scenes.uniform_soup(4096, seed=9)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    out, root, trace = orc.bittner_seq(nodes, 10)
    assert trace[-1] < trace[0] * 0.9
    assert orc.validate(out, vert, faces, root=root) == [0, 0, 0, 0, 0]


def test_bittner_chunked_improves_and_stays_valid(orc):
    vert, faces = scenes.uniform_soup(4096, seed=9)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    out, trace, st = orc.bittner_chunked(nodes, 10)
    assert np.all(np.diff(trace) <= 1e-9 * trace[0]) or trace[-1] < trace[0]
    assert trace[-1] < trace[0] * 0.9
    assert orc.validate(out, vert, faces) == [0, 0, 0, 0, 0]
    assert st["applied"] > 0 and st["items"] == 10 * (int(0.01 * out.shape[0]) // 32) * 32
    # deterministic
    out2, trace2, _ = orc.bittner_chunked(nodes, 10)
    assert np.array_equal(out.view(np.uint8), out2.view(np.uint8))


def test_batched_search_reaches_the_heap_order_sah(orc):
    """The batched search (whole-frontier rounds) finds the same optimum as the reference's
    heap order up to ties and overflow: equal iteration counts give SAH within 0.5%."""
    vert, faces = scenes.uniform_soup(20000, seed=21)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    _, tb, st_b = orc.bittner_chunked(nodes, 10, search_mode=0)
    _, th, _ = orc.bittner_chunked(nodes, 10, search_mode=1)
    assert abs(tb[-1] / th[-1] - 1.0) <= 0.005, (tb[-1], th[-1])
    assert tb[-1] < 0.8 * tb[0]


@pytest.mark.parametrize("offset_access", [False, True])
def test_ordered_iteration_reads_only_the_batch_prefix(orc, offset_access):
    """A chunked iteration processes the positions below numChunks * chunkSize of its order (in
    chunk-major or strided batch order), so that prefix gives the same tree as the whole order:
    the GPU selection keeps only the prefix."""
    vert, faces = scenes.uniform_soup(6000, seed=4)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    inner = np.nonzero(nodes["isLeafFlag"] == 0)[0].astype(np.uint32)
    order = np.random.default_rng(3).permutation(inner).astype(np.uint32)
    k = int(0.01 * nodes.shape[0]) // 32 * 32
    assert 0 < k < order.shape[0]
    a = np.ascontiguousarray(nodes.copy())
    b = np.ascontiguousarray(nodes.copy())
    sa = orc.bittner_iteration_ordered(a, order, offset_access=offset_access)
    sb = orc.bittner_iteration_ordered(b, order[:k], offset_access=offset_access)
    assert sa == sb and sa["items"] == k
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
