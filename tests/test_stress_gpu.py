"""Combined stress scene at full size (33,554,432 triangles: 512 rotated, tessellated boxes and a
256-component Gaussian mixture), checked through properties that do not depend on the size:

* the scene box and a sample of 63-bit Morton codes equal the oracle's;
* the sorted keys are ascending and stable, and equal the unsorted keys gathered by the order;
* every sampled inner node splits its leaf range exactly where the Karras rule puts it (the one
  adjacent pair whose common prefix equals the range's) and carries the Karras node index;
* after plain and learned Bittner13 iterations the tree passes the oracle's validator (structure,
  boxes, surface areas, triangles) and the GPU SAH equals the oracle's;
* the 16 incoherent ray batches (64k to 4M rays) give the oracle's closest hits on samples.
"""
import numpy as np
import pytest

from bvhtest_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def stress(gpu):
    import torch
    vert, faces = scenes.stress_scene()
    n = faces.shape[0]
    st = {"vert": vert, "faces": faces, "n": n,
          "v": torch.from_numpy(vert).cuda(), "f": torch.from_numpy(faces.view(np.int32)).cuda()}
    st["lbvh"] = gpu.LBVH(n, 63, "karras")
    st["nodes"] = st["lbvh"].build(st["v"], st["f"])
    torch.cuda.synchronize()
    yield st
    st["lbvh"].close()


def _clz64(x):
    """Leading zeros of non-zero uint64 values (binary search on the top bits)."""
    x = x.astype(np.uint64)
    n = np.zeros(x.shape, np.int64)
    for s in (32, 16, 8, 4, 2, 1):
        top_zero = x < (np.uint64(1) << np.uint64(64 - s))
        n += np.where(top_zero, s, 0)
        x = np.where(top_zero, x << np.uint64(s), x)
    return n


def _delta(keys, i, j):
    """delta of the 63-bit karras mode: clz64 of the keys' xor, 64 + clz32 of the indices' on ties."""
    x = keys[i] ^ keys[j]
    out = np.empty(i.shape[0], np.int64)
    nz = x != 0
    out[nz] = _clz64(x[nz])
    out[~nz] = 64 + _clz64((i ^ j)[~nz].astype(np.uint64)) - 32
    return out


def _descend(nodes, start, first_child, last_child="left"):
    """From each start node follow first_child once, then last_child down to a leaf."""
    cur = start if first_child is None else nodes[first_child][start].astype(np.int64)
    for _ in range(512):
        leaf = nodes["isLeafFlag"][cur] != 0
        if leaf.all():
            return cur
        cur = np.where(leaf, cur, nodes[last_child][cur].astype(np.int64))
    raise AssertionError("no leaf within 512 levels")


def test_stress_build_matches_the_oracle_on_size_independent_properties(gpu, orc, stress):
    n, vert, faces, lbvh = stress["n"], stress["vert"], stress["faces"], stress["lbvh"]
    assert n == 33554432 and lbvh.errors() == 0
    _, cen, scene = orc.tri_data(vert, faces)
    assert np.array_equal(lbvh.scene_box(), scene)
    keys, _ = lbvh.keys(n, False)
    g = np.random.default_rng(5)
    sample = g.choice(n, 200000, replace=False)
    assert np.array_equal(keys[sample], orc.morton(cen[sample], scene, 63))
    del cen
    sk, sidx = lbvh.keys(n, True)
    assert np.all(sk[1:] >= sk[:-1])
    ties = sk[1:] == sk[:-1]
    assert np.all(sidx[1:][ties] > sidx[:-1][ties])  # stable
    assert np.array_equal(sk, keys[sidx])

    nodes = gpu.nodes_to_numpy(stress["nodes"])[: 2 * n - 1]
    assert orc.validate(nodes, vert, faces)[:5] == [0, 0, 0, 0, 0]
    # leaf ranges of sampled inner nodes (leftmost and rightmost leaf) and the split (the left
    # child's rightmost leaf)
    inner = g.choice(n - 1, 20000, replace=False).astype(np.int64)
    l = _descend(nodes, inner, None, "left") - (n - 1)
    r = _descend(nodes, inner, None, "right") - (n - 1)
    split = _descend(nodes, inner, "left", "right") - (n - 1)
    assert np.all((l >= 0) & (l <= split) & (split < r) & (r < n))
    assert np.array_equal(_delta(sk, split, split + 1), _delta(sk, l, r))
    # Karras numbering: a left child is numbered by its last leaf, a right child by its first
    root = inner == 0
    is_left = nodes["isLeft"][inner] != 0
    assert np.all(root | (inner == np.where(is_left, r, l)))
    assert np.all((l[root] == 0) & (r[root] == n - 1))


def test_stress_optimizer_keeps_a_valid_tree(gpu, orc, stress):
    import torch
    n, nodes = stress["n"], stress["nodes"]
    opt = gpu.Bittner13GPU(nodes, num_nodes=2 * n - 1)
    opt.set_scorer(gpu.Mlp(seed=3), 2)  # learned and plain iterations alternate; weights do not matter here
    before = gpu.calc_sah(nodes, 0, 2 * n - 1)
    opt.run(4)
    torch.cuda.synchronize()
    st = opt.stats()  # raises if a kernel flagged an error
    assert st["applied"] > 0
    host = gpu.nodes_to_numpy(nodes)[: 2 * n - 1]
    assert orc.validate(host, stress["vert"], stress["faces"])[:5] == [0, 0, 0, 0, 0]
    sah = gpu.calc_sah(nodes, 0, 2 * n - 1)
    assert abs(sah - orc.sah(host)) <= 1e-6 * sah
    assert sah < before
    opt.close()
    stress["host"] = host


def test_stress_ray_batches_match_the_oracle(gpu, orc, stress):
    n, vert, faces = stress["n"], stress["vert"], stress["faces"]
    host = stress.get("host")
    if host is None:
        host = gpu.nodes_to_numpy(stress["nodes"])[: 2 * n - 1]
    org, dirs, sizes = scenes.stress_rays(vert.min(0), vert.max(0))
    assert len(sizes) == 16 and sum(sizes) == 16777216 and min(sizes) == 65536 and max(sizes) == 4194304
    g = np.random.default_rng(9)
    off = 0
    hit_total = 0
    for sz in sizes:
        sl = slice(off, off + sz)
        h = gpu.hits_to_numpy(gpu.trace_rays(stress["nodes"], stress["v"], stress["f"], org[sl], dirs[sl],
                                             num_nodes=2 * n - 1))
        hit_total += int((h["prim"] != 0xFFFFFFFF).sum())
        pick = g.choice(sz, 512, replace=False)
        ref = orc.trace_bvh(org[sl][pick], dirs[sl][pick], host, vert, faces)
        assert np.array_equal(h["prim"][pick], ref["prim"])
        hit = ref["prim"] != 0xFFFFFFFF
        assert np.allclose(h["t"][pick][hit], ref["t"][hit], rtol=1e-5, atol=0)
        off += sz
    assert gpu.trace_errors() == 0
    assert hit_total > 0.2 * sum(sizes)  # about 38% of these rays meet a surface
