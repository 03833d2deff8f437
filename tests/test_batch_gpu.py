"""Batched multi-mesh pipeline: every mesh's result must equal the single-mesh pipeline on that mesh.

Meshes of uneven size (including 1, 2 and 3 triangles) are concatenated; the batched LBVH, Bittner13
iterations and random-ray trace are compared byte for byte with bvhgb_lbvh_build, bvhgb_bn13_run and
bvhgb_trace_rays run on each mesh alone, and the tracer's hits with the oracle's brute force. The
captured graph must reproduce the step-by-step results, and every autotuner configuration the same.
"""
import numpy as np
import pytest

from bvhtest_gb300 import scenes

pytestmark = pytest.mark.gpu
COUNTS = [1, 2, 3, 17, 500, 4096, 1, 20000, 777, 9000]


def _scene(counts, seed=5):
    verts, faces, base = [], [], 0
    for m, n in enumerate(counts):
        v, _ = scenes.gmm_soup(n, clusters=1 + m % 7, seed=seed * 100 + m, extent=1.0, sigma_lo=0.005,
                               sigma_hi=0.08, vertex_sigma=0.004)
        verts.append(v.reshape(-1, 3))
        faces.append(np.arange(3 * n, dtype=np.uint32).reshape(n, 3) + base)
        base += 3 * n
    return np.concatenate(verts).astype(np.float32), np.concatenate(faces).astype(np.uint32)


def _dev(vert, faces):
    import torch
    return torch.from_numpy(vert).cuda(), torch.from_numpy(faces.view(np.int32)).cuda()


def _mesh(vert, faces, fo, m):
    """Mesh m alone: its vertices and faces renumbered from 0."""
    f = faces[fo[m]:fo[m + 1]]
    lo = int(f.min()) if len(f) else 0
    return vert[lo: int(f.max()) + 1 if len(f) else 0], (f - lo).astype(np.uint32)


@pytest.mark.parametrize("topo", ["refCompat", "karras"])
def test_batched_build_equals_single_mesh_builds(gpu, topo):
    import torch
    vert, faces = _scene(COUNTS)
    v, f = _dev(vert, faces)
    b = gpu.Batch(COUNTS, topology=topo)
    nodes = b.empty_nodes()
    b.build(v, f, nodes)
    torch.cuda.synchronize()
    for m, n in enumerate(COUNTS):
        mv, mf = _mesh(vert, faces, b.face_offsets, m)
        ref = gpu.LBVH(n, 30, topo).build(*_dev(mv, mf))
        got = b.mesh_nodes(nodes, m)
        assert torch.equal(got, ref[: 2 * n - 1]), (m, n)
    assert b.stats()[1] == 0


def test_batched_optimizer_and_trace_equal_single_mesh(gpu, orc):
    import torch
    vert, faces = _scene(COUNTS, seed=6)
    v, f = _dev(vert, faces)
    b = gpu.Batch(COUNTS)
    nodes = b.empty_nodes()
    b.build(v, f, nodes)
    b.optimize(nodes, 4)
    hits, org, dirs = b.trace_random(nodes, v, f, 512, seed=7, with_rays=True)
    torch.cuda.synchronize()
    st, err = b.stats()
    assert err == 0 and st["applied"] > 0
    for m, n in enumerate(COUNTS):
        mv, mf = _mesh(vert, faces, b.face_offsets, m)
        dv, df = _dev(mv, mf)
        ref = gpu.LBVH(n, 30).build(dv, df)
        if n > 1:
            opt = gpu.Bittner13GPU(ref, num_nodes=2 * n - 1)
            opt.run(4)
        got = b.mesh_nodes(nodes, m)
        assert torch.equal(got, ref[: 2 * n - 1]), (m, n)
        sl = slice(m * 512, (m + 1) * 512)
        single = gpu.trace_rays(ref, dv, df, org[sl], dirs[sl], num_nodes=2 * n - 1)
        assert torch.equal(hits[sl], single), m
        if n <= 4096:
            bf = orc.trace_brute(org[sl].cpu().numpy(), dirs[sl].cpu().numpy(), mv, mf)
            h = gpu.hits_to_numpy(hits[sl])
            assert np.array_equal(h["prim"], bf["prim"]), m
    # the rays start inside each mesh's box grown 1.5x and point in unit directions
    assert torch.allclose(dirs.norm(dim=1), torch.ones(dirs.shape[0], device="cuda"), atol=1e-5)


def test_captured_graph_and_every_tuning_give_the_same_result(gpu):
    import torch
    vert, faces = _scene(COUNTS, seed=8)
    v, f = _dev(vert, faces)
    b = gpu.Batch(COUNTS)
    ref = b.empty_nodes()
    b.build(v, f, ref)
    b.optimize(ref, 3)
    ref_hits = b.trace_random(ref, v, f, 256, seed=3)
    nodes = b.empty_nodes()
    hits = torch.empty_like(ref_hits)
    b.run(v, f, nodes, 3, 256, hits, seed=3)
    b.run(v, f, nodes, 3, 256, hits, seed=3)  # replay of the captured graph
    torch.cuda.synchronize()
    assert torch.equal(nodes, ref) and torch.equal(hits, ref_hits)
    for tile in (2048, 4096, 8192):
        for blk in (128, 512):
            b.set_config(sortTileKeys=tile, refitBlock=blk, traceBlock=64 if blk == 128 else 256)
            n2 = b.empty_nodes()
            h2 = torch.empty_like(ref_hits)
            b.run(v, f, n2, 3, 256, h2, seed=3)
            torch.cuda.synchronize()
            assert torch.equal(n2, ref) and torch.equal(h2, ref_hits), (tile, blk)
    rep = b.autotune(v, f, nodes, 256, hits, seed=3)
    assert sorted(rep["sort_tile"]) == [2048, 4096, 8192] and len(rep["refit_block"]) == 3
    assert rep["chosen"]["sortTileKeys"] in (2048, 4096, 8192)
    assert all(t > 0 for t in rep["sort_tile"].values())
    b.run(v, f, nodes, 3, 256, hits, seed=3)
    torch.cuda.synchronize()
    assert torch.equal(nodes, ref) and torch.equal(hits, ref_hits)


def test_batch_rejects_bad_arguments(gpu):
    with pytest.raises(gpu.BvhgbError):
        gpu.Batch([10, 20], sort_tile=1000)
    b = gpu.Batch([10, 0, 20])
    import torch
    vert, faces = _scene([10, 20])
    v, f = _dev(vert, faces)
    nodes = b.empty_nodes()
    b.build(v, f, nodes)  # an empty mesh builds to nothing
    with pytest.raises(gpu.BvhgbError):
        b.trace_random(nodes, v, f, 16)  # but cannot be traced
