"""GPU parity of the LBVH build and the radix sort against the oracle (bit-exact)."""
import json
from pathlib import Path

import numpy as np
import pytest

from bvhtest_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _dev(gpu, vert, faces):
    import torch
    return (torch.from_numpy(vert).cuda(), torch.from_numpy(faces.view(np.int32)).cuda())


@pytest.mark.parametrize("n", [1, 2, 3, 5, 64, 1000, 4097, 65536, (1 << 20) + 7])
@pytest.mark.parametrize("bits,topo", [(30, "refCompat"), (30, "karras"), (63, "karras"), (63, "refCompat")])
def test_lbvh_bit_exact(gpu, orc, n, bits, topo):
    import torch
    if n > 100000 and (bits, topo) == (63, "refCompat"):
        pytest.skip("covered at smaller sizes")
    vert, faces = scenes.uniform_soup(n, seed=n + bits)
    v, f = _dev(gpu, vert, faces)
    b = gpu.LBVH(n, bits, topo)
    # phases: scene box, Morton codes, sorted order
    b.init_tri_data(v, f)
    b.calc_morton(v, f)
    b.sort(n)
    nodes = gpu.empty_nodes(2 * n - 1)
    b.build_tree(v, f, nodes)
    torch.cuda.synchronize()
    _, cen, scene = orc.tri_data(vert, faces)
    assert np.array_equal(b.scene_box(), scene)
    k_gpu, _ = b.keys(n, False)
    assert np.array_equal(k_gpu, orc.morton(cen, scene, bits))
    ref_nodes, ref_keys, ref_idx = orc.lbvh_build(vert, faces, bits, 0 if topo == "refCompat" else 1)
    ks, idx = b.keys(n, True)
    assert np.array_equal(ks, ref_keys)
    assert np.array_equal(idx, ref_idx)
    got = gpu.nodes_to_numpy(nodes)[: 2 * n - 1]
    assert np.array_equal(got.view(np.uint8), ref_nodes.view(np.uint8)), _first_diff(got, ref_nodes)
    assert b.errors() == 0
    # a second build_tree from the same sorted keys re-arms its exchange slots
    b.build_tree(v, f, nodes)
    torch.cuda.synchronize()
    assert np.array_equal(gpu.nodes_to_numpy(nodes)[: 2 * n - 1].view(np.uint8), ref_nodes.view(np.uint8))
    # whole-command entry point gives the same bytes
    nodes2 = b.build(v, f)
    assert np.array_equal(gpu.nodes_to_numpy(nodes2)[: 2 * n - 1].view(np.uint8), ref_nodes.view(np.uint8))
    b.close()


def _first_diff(a, b):
    d = np.nonzero(a.view(np.uint8).reshape(len(a), 48) != b.view(np.uint8).reshape(len(b), 48))
    if len(d[0]) == 0:
        return "equal"
    i = d[0][0]
    return f"node {i}: gpu {a[i]} vs oracle {b[i]}"


def test_lbvh_matches_committed_fixture(gpu):
    import torch
    g = np.load(GOLDEN / "oracle_small.npz")
    for n in (257, 1000):
        vert = g[f"n{n}_vert"]
        faces = np.arange(3 * n, dtype=np.uint32).reshape(-1, 3)
        v, f = _dev(gpu, vert, faces)
        for bits in (30, 63):
            for topo, name in (("refCompat", "ref"), ("karras", "kar")):
                b = gpu.LBVH(n, bits, topo)
                nodes = b.build(v, f)
                torch.cuda.synchronize()
                assert np.array_equal(gpu.nodes_to_numpy(nodes)[: 2 * n - 1].view(np.uint8),
                                      g[f"n{n}_b{bits}_{name}_nodes"])
                sah = gpu.calc_sah(nodes, 0, 2 * n - 1)
                assert abs(sah - float(g[f"n{n}_b{bits}_{name}_sah"])) <= 1e-9 * sah
                b.close()


def test_lbvh_large_properties(gpu, orc):
    """4,194,304 triangles, 63-bit keys: size-independent checks (sorted keys, permutation,
    Validate invariants, SAH against the oracle)."""
    import torch
    vert, faces = scenes.large_scene()
    n = faces.shape[0]
    v, f = _dev(gpu, vert, faces)
    b = gpu.LBVH(n, 63, "karras")
    nodes = b.build(v, f)
    torch.cuda.synchronize()
    ks, idx = b.keys(n, True)
    assert np.all(ks[1:] >= ks[:-1])
    assert np.array_equal(np.sort(idx), np.arange(n, dtype=np.uint32))
    got = gpu.nodes_to_numpy(nodes)
    assert orc.validate(got, vert, faces) == [0, 0, 0, 0, 0]
    ref_nodes, _, _ = orc.lbvh_build(vert, faces, 63, 1)
    assert np.array_equal(got.view(np.uint8), ref_nodes.view(np.uint8))


def test_lbvh_reuse_and_errors(gpu):
    import torch
    vert, faces = scenes.uniform_soup(100, seed=1)
    v, f = _dev(gpu, vert, faces)
    b = gpu.LBVH(100)
    first = gpu.nodes_to_numpy(b.build(v, f))
    second = gpu.nodes_to_numpy(b.build(v, f))
    assert np.array_equal(first.view(np.uint8), second.view(np.uint8))
    vert2, faces2 = scenes.uniform_soup(200, seed=2)
    v2, f2 = _dev(gpu, vert2, faces2)
    with pytest.raises(gpu.BvhgbError):
        b.build(v2, f2)  # more faces than the workspace was created for
    with pytest.raises(gpu.BvhgbError):
        gpu.LBVH(10, morton_bits=31)
    torch.cuda.synchronize()


@pytest.mark.parametrize("n", [0, 1, 31, 4096, 4097, 100000, 3000001])
@pytest.mark.parametrize("width", [32, 64])
def test_radix_sort_stable(gpu, n, width):
    import torch
    g = np.random.default_rng(n + width)
    if width == 32:
        keys = g.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
        if n > 10:
            keys[: n // 3] = keys[0]  # many duplicates
        kt = torch.from_numpy(keys.view(np.int32)).cuda()
    else:
        keys = g.integers(0, 1 << 63, n, dtype=np.uint64)
        if n > 10:
            keys[n // 2:] &= np.uint64(0xFF)
        kt = torch.from_numpy(keys.view(np.int64)).cuda()
    vals = np.arange(n, dtype=np.uint32)
    vt = torch.from_numpy(vals.view(np.int32)).cuda()
    ko, vo = gpu.radix_sort_pairs(kt, vt)
    torch.cuda.synchronize()
    order = np.argsort(keys, kind="stable")
    got_k = ko.cpu().numpy().view(keys.dtype)
    got_v = vo.cpu().numpy().view(np.uint32)
    assert np.array_equal(got_k, keys[order])
    assert np.array_equal(got_v, vals[order])


def test_radix_sort_bit_range(gpu):
    import torch
    g = np.random.default_rng(1)
    keys = g.integers(0, 1 << 30, 50000, dtype=np.uint64).astype(np.uint32)
    kt = torch.from_numpy(keys.view(np.int32)).cuda()
    vt = torch.arange(50000, dtype=torch.int32, device="cuda")
    ko, vo = gpu.radix_sort_pairs(kt, vt, 8, 20)
    torch.cuda.synchronize()
    digit = (keys >> 8) & ((1 << 12) - 1)
    order = np.argsort(digit, kind="stable")
    assert np.array_equal(vo.cpu().numpy(), order)


@pytest.mark.parametrize("tile", [2048, 4096, 8192])
def test_sort_default_tile_gives_the_same_order(gpu, tile):
    import torch
    g = np.random.default_rng(tile)
    n = 1000003
    keys = g.integers(0, 1 << 63, n, dtype=np.uint64)
    keys[::3] = keys[7]  # runs of equal keys keep their input order
    kt = torch.from_numpy(keys.view(np.int64)).cuda()
    vt = torch.arange(n, dtype=torch.int32, device="cuda")
    prev = gpu.sort_default_tile(tile)
    try:
        assert gpu.sort_default_tile(0) == tile
        ko, vo = gpu.radix_sort_pairs(kt, vt)
        torch.cuda.synchronize()
    finally:
        gpu.sort_default_tile(prev)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(vo.cpu().numpy().view(np.uint32), order.astype(np.uint32))
    assert np.array_equal(ko.cpu().numpy().view(np.uint64), keys[order])
    with pytest.raises(gpu.BvhgbError):
        gpu.sort_default_tile(1000)


@pytest.mark.parametrize("n,k,kind", [(1, 1, "random"), (5000, 1, "random"), (5000, 4999, "ties"),
                                      (5000, 5000, "random"), (100003, 1000, "ties"), (100003, 77777, "equal"),
                                      (4194303, 83872, "random"), (4194303, 83872, "ties"), (1000000, 83872, "few")])
def test_select_smallest_is_the_stable_sort_prefix(gpu, n, k, kind):
    """The k smallest keys' values in stable ascending order equal the first k of the full stable sort,
    with runs of equal keys cut at k in index order."""
    import torch
    g = np.random.default_rng(n + k)
    if kind == "random":
        keys = g.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    elif kind == "ties":
        keys = g.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
        keys[: n // 2] = keys[0]
    elif kind == "equal":
        keys = np.full(n, 0x3F800000, np.uint32)
    else:  # few distinct values that share their high digits
        keys = (g.integers(0, 4, n).astype(np.uint32) << 21) | g.integers(0, 3, n).astype(np.uint32)
    vals = g.permutation(n).astype(np.uint32)
    kt = torch.from_numpy(keys.view(np.int32)).cuda()
    vt = torch.from_numpy(vals.view(np.int32)).cuda()
    out = gpu.select_smallest_pairs(kt, vt, k)
    torch.cuda.synchronize()
    want = vals[np.argsort(keys, kind="stable")[:k]]
    assert np.array_equal(out.cpu().numpy().view(np.uint32), want)


def test_select_smallest_on_an_unaligned_key_array(gpu):
    """Keys that start 4 bytes past a 16-byte boundary take the scalar loads: same result."""
    import torch
    g = np.random.default_rng(77)
    n, k = 300001, 5000
    keys = g.integers(0, 1 << 32, n + 1, dtype=np.uint64).astype(np.uint32)
    vals = g.permutation(n + 1).astype(np.uint32)
    kt = torch.from_numpy(keys.view(np.int32)).cuda()[1:]
    vt = torch.from_numpy(vals.view(np.int32)).cuda()[1:]
    assert kt.data_ptr() % 16 == 4
    out = gpu.select_smallest_pairs(kt, vt, k)
    torch.cuda.synchronize()
    want = vals[1:][np.argsort(keys[1:], kind="stable")[:k]]
    assert np.array_equal(out.cpu().numpy().view(np.uint32), want)
