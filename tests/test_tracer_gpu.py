"""GPU parity of the closest-hit tracer: hit IDs and t bit-exact against the oracle's watertight
brute force (and its conservative BVH traversal, which the CPU tests pin to brute force)."""
import numpy as np
import pytest

from bvhtest_gb300 import scenes

pytestmark = pytest.mark.gpu
MISS = 0xFFFFFFFF


def _scene(gpu, n, seed=1, bits=30, topo="refCompat"):
    import torch
    vert, faces = scenes.uniform_soup(n, seed=seed)
    v = torch.from_numpy(vert).cuda()
    f = torch.from_numpy(faces.view(np.int32)).cuda()
    b = gpu.LBVH(n, bits, topo)
    nodes = b.build(v, f)
    torch.cuda.synchronize()
    return vert, faces, v, f, nodes


def test_primary_image_matches_oracle(gpu, orc):
    import torch
    vert, faces, v, f, nodes = _scene(gpu, 65536)
    cam = scenes.camera_default()
    gpu.trace_errors(reset=True)
    img, hits = gpu.trace_image(nodes, v, f, cam)
    torch.cuda.synchronize()
    assert gpu.trace_errors() == 0
    h = gpu.hits_to_numpy(hits)
    px = gpu.pixels_to_numpy(img)
    org, dirs = orc.camera_rays(cam["pos"], cam["lookAt"], cam["up"], cam["fov"], cam["width"], cam["height"])
    ref = orc.trace_bvh(org, dirs, gpu.nodes_to_numpy(nodes), vert, faces)
    assert np.array_equal(h["prim"], ref["prim"])
    hit = ref["prim"] != MISS
    assert hit.mean() > 0.1  # the 65,536 tiny triangles cover about 13% of this view
    assert np.array_equal(h["t"][hit], ref["t"][hit])
    # brute force on every 61st pixel
    sel = np.arange(0, org.shape[0], 61)
    bf = orc.trace_brute(org[sel], dirs[sel], vert, faces)
    assert np.array_equal(h["prim"][sel], bf["prim"])
    # shading of the CUDAPixel image
    assert np.array_equal(px["hit"], hit.astype(np.uint8))
    for i in np.nonzero(hit)[0][::97]:
        tri = faces[h["prim"][i]]
        d = orc.shade(org[i], dirs[i], h["t"][i], vert[tri[0]], vert[tri[1]], vert[tri[2]])
        assert px["diffuse"][i] == d
    assert px["intCount"].max() > 0


@pytest.mark.parametrize("topo", ["refCompat", "karras"])
def test_random_rays_match_oracle(gpu, orc, topo):
    import torch
    vert, faces, v, f, nodes = _scene(gpu, 20000, seed=3, topo=topo)
    org, dirs = scenes.random_rays(50000, (-0.25, -0.25, -0.25), (1.25, 1.25, 1.25), seed=4)
    hits = gpu.trace_rays(nodes, v, f, org, dirs)
    torch.cuda.synchronize()
    h = gpu.hits_to_numpy(hits)
    ref = orc.trace_bvh(org, dirs, gpu.nodes_to_numpy(nodes), vert, faces)
    assert np.array_equal(h["prim"], ref["prim"])
    hit = ref["prim"] != MISS
    assert np.array_equal(h["t"][hit], ref["t"][hit])
    bf = orc.trace_brute(org[:2000], dirs[:2000], vert, faces)
    assert np.array_equal(h["prim"][:2000], bf["prim"])


def test_face_culling_and_t_range(gpu, orc):
    import torch
    vert, faces, v, f, nodes = _scene(gpu, 5000, seed=5)
    org, dirs = scenes.random_rays(5000, (0, 0, 0), (1, 1, 1), seed=6)
    for cull, tmin, tmax in ((True, 0.0, np.inf), (False, 0.1, 0.5)):
        hits = gpu.trace_rays(nodes, v, f, org, dirs, tmin=tmin, tmax=tmax, face_culling=cull)
        torch.cuda.synchronize()
        h = gpu.hits_to_numpy(hits)
        bf = orc.trace_brute(org, dirs, vert, faces, tmin=tmin, tmax=tmax, cull=cull)
        assert np.array_equal(h["prim"], bf["prim"])


def test_axis_parallel_and_edge_rays(gpu, orc):
    import torch
    # a 2x2 grid of quads (8 triangles sharing edges and vertices) in the z = 0.5 plane
    pts = []
    for i in range(2):
        for j in range(2):
            a, b, c, d = (i, j), (i + 1, j), (i + 1, j + 1), (i, j + 1)
            pts += [a, b, c, a, c, d]
    vert = np.array([[x * 0.5, y * 0.5, 0.5] for x, y in pts], np.float32)
    faces = np.arange(len(vert), dtype=np.uint32).reshape(-1, 3)
    v = torch.from_numpy(vert).cuda()
    f = torch.from_numpy(faces.view(np.int32)).cuda()
    b = gpu.LBVH(faces.shape[0])
    nodes = b.build(v, f)
    # rays along +z / -z through interior points, shared edges and shared vertices
    xs = np.linspace(0.0, 1.0, 9, dtype=np.float32)
    grid = np.array([[x, y] for x in xs for y in xs], np.float32)
    org = np.concatenate([np.c_[grid, np.zeros(len(grid))], np.c_[grid, np.ones(len(grid))]]).astype(np.float32)
    dirs = np.concatenate([np.tile([0, 0, 1], (len(grid), 1)), np.tile([0, 0, -1], (len(grid), 1))]).astype(np.float32)
    hits = gpu.trace_rays(nodes, v, f, org, dirs)
    torch.cuda.synchronize()
    h = gpu.hits_to_numpy(hits)
    bf = orc.trace_brute(org, dirs, vert, faces)
    assert np.array_equal(h["prim"], bf["prim"])
    inside = (org[:, 0] > 0) & (org[:, 0] < 1) & (org[:, 1] > 0) & (org[:, 1] < 1)
    assert np.all(h["prim"][inside] != MISS)  # watertight: no ray escapes through an edge


def test_bounce_rays_match_oracle(gpu, orc):
    """Cosine-weighted bounce rays: the GPU reports the rays it generated; the oracle traces those
    same rays and must find the same closest hits."""
    import torch
    vert, faces, v, f, nodes = _scene(gpu, 65536, seed=9, topo="karras")
    cam = dict(scenes.camera_default(), width=256, height=192)
    _, hits = gpu.trace_image(nodes, v, f, cam)
    bounce, org, dirs = gpu.trace_bounce(nodes, v, f, cam, hits, seed=7, with_rays=True)
    torch.cuda.synchronize()
    ph = gpu.hits_to_numpy(hits)
    bh = gpu.hits_to_numpy(bounce)
    org, dirs = org.cpu().numpy(), dirs.cpu().numpy()
    live = ph["prim"] != MISS
    assert live.sum() > 1000
    assert np.all(bh["prim"][~live] == MISS)
    ref = orc.trace_bvh(org[live], dirs[live], gpu.nodes_to_numpy(nodes), vert, faces)
    assert np.array_equal(bh["prim"][live], ref["prim"])
    # bounce directions are unit length and leave the surface on the camera's side
    assert np.allclose(np.linalg.norm(dirs[live], axis=1), 1.0, atol=1e-5)
    assert (bh["prim"][live] != MISS).mean() > 0.05


def test_rays_missing_everything(gpu):
    import torch
    vert, faces, v, f, nodes = _scene(gpu, 1000, seed=8)
    org = np.tile(np.float32([5, 5, 5]), (100, 1))
    dirs = np.tile(np.float32([0, 0, 1]), (100, 1))
    h = gpu.hits_to_numpy(gpu.trace_rays(nodes, v, f, org, dirs))
    torch.cuda.synchronize()
    assert np.all(h["prim"] == MISS) and np.all(np.isinf(h["t"]))


def test_prepared_tracer_gives_the_same_hits(gpu):
    """bvhgb_tracer_*: the traversal records (both children per record) give the node-array
    traversal's hits for primary, bounce and random rays, and again after the tree changes."""
    import torch
    vert, faces, v, f, nodes = _scene(gpu, 20000, seed=4, bits=63, topo="karras")
    n_nodes = 2 * 20000 - 1
    tr = gpu.Tracer(n_nodes).update(nodes, num_nodes=n_nodes)
    cam = scenes.camera_default()
    for round_ in range(2):
        img_a, hits_a = gpu.trace_image(nodes, v, f, cam, num_nodes=n_nodes)
        img_b, hits_b = tr.trace_image(v, f, cam)
        bounce_a, _, _ = gpu.trace_bounce(nodes, v, f, cam, hits_a, seed=3, num_nodes=n_nodes)
        bounce_b, _, _ = tr.trace_bounce(v, f, cam, hits_b, seed=3)
        org, dirs = scenes.random_rays(8192, vert.min(0), vert.max(0), seed=5 + round_)
        rays_a = gpu.trace_rays(nodes, v, f, org, dirs, num_nodes=n_nodes)
        rays_b = tr.trace_rays(v, f, org, dirs)
        torch.cuda.synchronize()
        assert torch.equal(hits_a, hits_b) and torch.equal(bounce_a, bounce_b) and torch.equal(rays_a, rays_b)
        px_a, px_b = gpu.pixels_to_numpy(img_a), gpu.pixels_to_numpy(img_b)
        assert np.array_equal(px_a["hit"], px_b["hit"]) and np.array_equal(px_a["diffuse"], px_b["diffuse"])
        assert (gpu.hits_to_numpy(rays_a)["prim"] != MISS).mean() > 0.05  # about 11% of these rays hit
        if round_ == 0:  # change the tree, rebuild the records
            opt = gpu.Bittner13GPU(nodes, num_nodes=n_nodes)
            opt.run(3)
            opt.close()
            tr.update(nodes, num_nodes=n_nodes)
    assert gpu.trace_errors() == 0
    tr.close()


@pytest.mark.parametrize("cull", [False, True])
def test_ray_bundles_give_the_per_ray_hits(gpu, orc, cull):
    """rayBundles (the reference's kTraceRayBundle, CUDAKernels.cu:240-383): a warp of neighbouring
    primary rays traverses as one bundle; every ray still gets the closest hit of its own
    traversal (and of the brute force), on the node array and on the traversal records, for a
    camera whose image edges leave partial warps."""
    import torch
    vert, faces, v, f, nodes = _scene(gpu, 30000, seed=9)
    n_nodes = 2 * 30000 - 1
    cam = dict(scenes.camera_default(), width=203, height=117)
    tr = gpu.Tracer(n_nodes).update(nodes, num_nodes=n_nodes)
    img_a, hits_a = gpu.trace_image(nodes, v, f, cam, num_nodes=n_nodes, face_culling=cull)
    img_b, hits_b = gpu.trace_image(nodes, v, f, cam, num_nodes=n_nodes, face_culling=cull, ray_bundles=True)
    img_c, hits_c = tr.trace_image(v, f, cam, face_culling=cull, ray_bundles=True)
    torch.cuda.synchronize()
    assert gpu.trace_errors() == 0
    assert torch.equal(hits_a, hits_b) and torch.equal(hits_a, hits_c)
    pa, pb, pc = (gpu.pixels_to_numpy(x) for x in (img_a, img_b, img_c))
    for p in (pb, pc):
        assert np.array_equal(pa["hit"], p["hit"]) and np.array_equal(pa["diffuse"], p["diffuse"])
    h = gpu.hits_to_numpy(hits_b)
    org, dirs = orc.camera_rays(cam["pos"], cam["lookAt"], cam["up"], cam["fov"], cam["width"], cam["height"])
    sel = np.arange(0, org.shape[0], 37)
    bf = orc.trace_brute(org[sel], dirs[sel], vert, faces, cull=cull)
    assert np.array_equal(h["prim"][sel], bf["prim"])
    assert (h["prim"] != MISS).mean() > 0.02  # about 4% of this view hits the 30,000 small triangles
    # a bundle visits at least the nodes of each of its rays' own traversals
    assert (pb["intCount"].astype(np.int64) >= pa["intCount"]).all()
    tr.close()
