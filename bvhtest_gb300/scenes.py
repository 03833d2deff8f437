"""Seeded synthetic scenes with the shapes and distributions of the benchmark configurations.

The reference's own mesh files are not available, so these generators stand in for them. Every
scene is a soup of independent fp32 triangles (three unique vertices each, faces = iota), drawn
from numpy's Philox counter-based generator so the same seed gives the same bytes on x86-64
and aarch64.
"""
from __future__ import annotations

import numpy as np


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(int(seed)))


def _soup(vert: np.ndarray):
    vert = np.ascontiguousarray(vert.reshape(-1, 3), dtype=np.float32)
    faces = np.arange(vert.shape[0], dtype=np.uint32).reshape(-1, 3)
    return vert, faces


def uniform_soup(n: int = 65536, sigma: float = 0.004, seed: int = 1):
    """Small plain-method scene: centroids uniform in [0,1]^3, each vertex = centroid + N(0, sigma^2)
    per axis (65,536 triangles by default)."""
    g = _rng(seed)
    c = g.random((n, 1, 3), dtype=np.float64).astype(np.float32)
    off = g.normal(0.0, sigma, (n, 3, 3)).astype(np.float32)
    return _soup(c + off)


def gmm_soup(n: int, clusters: int = 64, seed: int = 2, sigma_lo: float = 0.05, sigma_hi: float = 0.8,
             extent: float = 10.0, vertex_sigma: float = 0.01):
    """Isotropic Gaussian mixture: means uniform in [0, extent]^3, sigma log-uniform in
    [sigma_lo, sigma_hi]; each triangle = a centroid drawn from the mixture plus per-vertex
    N(0, vertex_sigma^2) offsets."""
    g = _rng(seed)
    means = g.random((clusters, 3)) * extent
    sig = np.exp(g.uniform(np.log(sigma_lo), np.log(sigma_hi), clusters))
    comp = g.integers(0, clusters, n)
    c = means[comp] + g.normal(0.0, 1.0, (n, 3)) * sig[comp, None]
    off = g.normal(0.0, vertex_sigma, (n, 3, 3))
    return _soup((c[:, None, :] + off).astype(np.float32))


def ground_grid(cells: int, size: float = 10.0):
    """cells x cells quads at y = 0 over [0, size]^2, two triangles each."""
    xs = np.linspace(0.0, size, cells + 1, dtype=np.float64)
    x0, z0 = np.meshgrid(xs[:-1], xs[:-1], indexing="ij")
    x1, z1 = np.meshgrid(xs[1:], xs[1:], indexing="ij")
    x0, z0, x1, z1 = (a.reshape(-1) for a in (x0, z0, x1, z1))
    y = np.zeros_like(x0)
    t1 = np.stack([np.stack([x0, y, z0], 1), np.stack([x1, y, z0], 1), np.stack([x1, y, z1], 1)], 1)
    t2 = np.stack([np.stack([x0, y, z0], 1), np.stack([x1, y, z1], 1), np.stack([x0, y, z1], 1)], 1)
    return np.concatenate([t1, t2], 0).astype(np.float32)


def large_scene(n: int = 4194304, seed: int = 2, grid_cells: int = 724):
    """Large single scene: a ground grid of grid_cells^2 * 2 triangles (724 -> 1,048,352, about 25%)
    plus a 64-component mixture filling the rest, 4,194,304 triangles in total."""
    grid = ground_grid(grid_cells)
    rest = n - grid.shape[0]
    g_vert, _ = gmm_soup(rest, 64, seed)
    vert = np.concatenate([g_vert.reshape(-1, 3, 3), grid], 0)
    return _soup(vert)


def camera_default():
    """Pinhole at (0.5, 0.5, -1.5) looking +z at (0.5, 0.5, 0), up +y, 60 degree vertical FOV,
    512 x 512 pixels."""
    return dict(pos=(0.5, 0.5, -1.5), lookAt=(0.5, 0.5, 0.0), up=(0.0, 1.0, 0.0), fov=60.0, width=512, height=512)


def random_rays(n: int, lo, hi, seed: int = 3):
    """Origins uniform in the box [lo, hi], directions uniform on the unit sphere."""
    g = _rng(seed)
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    org = lo + g.random((n, 3)) * (hi - lo)
    d = g.normal(0.0, 1.0, (n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return org.astype(np.float32), d.astype(np.float32)


def batch_meshes(count: int = 256, lo: int = 1024, hi: int = 524288, seed: int = 9, clusters=(1, 16),
                 sigma=(0.005, 0.08), vertex_sigma: float = 0.004):
    """Batched-build scenes: count meshes with log-uniform triangle counts in [lo, hi]; mesh m is a
    Gaussian mixture in the unit cube (1-16 clusters, means uniform in [0,1]^3, sigma log-uniform in
    the given range, per-vertex offsets N(0, vertex_sigma^2)) with its own seed. Returns
    (vert [sum 3n, 3] float32, faces [sum n, 3] uint32 indexing the concatenated vertices, counts)."""
    g = _rng(seed)
    counts = np.exp(g.uniform(np.log(lo), np.log(hi), count)).astype(np.int64).clip(lo, hi)
    verts, faces, base = [], [], 0
    for m, n in enumerate(counts.tolist()):
        k = int(g.integers(clusters[0], clusters[1] + 1))
        gm = _rng(seed * 1000003 + m)
        means = gm.random((k, 3))
        sig = np.exp(gm.uniform(np.log(sigma[0]), np.log(sigma[1]), k))
        comp = gm.integers(0, k, n)
        c = means[comp] + gm.normal(0.0, 1.0, (n, 3)) * sig[comp, None]
        v = (c[:, None, :] + gm.normal(0.0, vertex_sigma, (n, 3, 3))).astype(np.float32).reshape(-1, 3)
        verts.append(v)
        faces.append((np.arange(3 * n, dtype=np.uint32).reshape(n, 3) + base).astype(np.uint32))
        base += 3 * n
    return np.concatenate(verts), np.concatenate(faces), counts.astype(np.uint32)


def _cube_faces(cells: int) -> np.ndarray:
    """The six faces of the cube [-1, 1]^3, each cells x cells quads split into two triangles,
    as [6 * cells^2 * 2, 3, 3] float64 vertices (outward winding is not relied on)."""
    t = np.linspace(-1.0, 1.0, cells + 1)
    u0, v0 = np.meshgrid(t[:-1], t[:-1], indexing="ij")
    u1, v1 = np.meshgrid(t[1:], t[1:], indexing="ij")
    u0, v0, u1, v1 = (a.reshape(-1) for a in (u0, v0, u1, v1))
    quads = []
    for axis in range(3):
        a, b = [k for k in range(3) if k != axis]
        for side in (-1.0, 1.0):
            def pt(u, v):
                p = np.empty((u.shape[0], 3))
                p[:, axis] = side
                p[:, a] = u
                p[:, b] = v
                return p
            p00, p10, p11, p01 = pt(u0, v0), pt(u1, v0), pt(u1, v1), pt(u0, v1)
            quads.append(np.stack([p00, p10, p11], 1))
            quads.append(np.stack([p00, p11, p01], 1))
    return np.concatenate(quads, 0)


def _random_rotations(g: np.random.Generator, k: int) -> np.ndarray:
    """k rotation matrices from uniformly distributed unit quaternions."""
    q = g.normal(0.0, 1.0, (k, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)


def box_soup(boxes: int = 512, cells: int = 52, seed: int = 5, extent: float = 10.0,
             half_lo: float = 0.1, half_hi: float = 0.6):
    """boxes randomly rotated boxes, centres uniform in [0, extent]^3, half extents uniform in
    [half_lo, half_hi] per axis; every face tessellated into cells x cells quads of two triangles
    (512 boxes x 6 faces x 52^2 x 2 = 16,613,376 triangles by default). Returns [n, 3, 3] float32."""
    g = _rng(seed)
    unit = _cube_faces(cells)                       # [T, 3, 3]
    centre = g.random((boxes, 3)) * extent
    half = g.uniform(half_lo, half_hi, (boxes, 3))
    rot = _random_rotations(g, boxes)
    out = np.empty((boxes, unit.shape[0], 3, 3), np.float32)
    step = 32
    for b0 in range(0, boxes, step):  # scale the cube, then rotate and move it (32 boxes at a time)
        b1 = min(boxes, b0 + step)
        local = unit[None] * half[b0:b1, None, None, :]
        out[b0:b1] = np.einsum("btvk,bjk->btvj", local, rot[b0:b1]) + centre[b0:b1, None, None, :]
    return out.reshape(-1, 3, 3)


def stress_scene(n: int = 33554432, boxes: int = 512, cells: int = 52, clusters: int = 256, seed: int = 5):
    """Combined stress scene: the rotated, tessellated boxes of box_soup (16,613,376 triangles)
    and a clusters-component Gaussian mixture (means uniform in [0,10]^3, sigma log-uniform in
    [0.05, 0.8], per-vertex offsets N(0, 0.01^2)) filling the rest: 33,554,432 triangles."""
    bx = box_soup(boxes, cells, seed)
    rest = n - bx.shape[0]
    if rest < 0:
        raise ValueError("the boxes alone exceed n")
    g_vert, _ = gmm_soup(rest, clusters, seed + 1)
    return _soup(np.concatenate([g_vert.reshape(-1, 3, 3), bx], 0))


# 16 ray batches of the stress test, in units of 65,536 rays: 64k up to 4M, 16,777,216 in total.
STRESS_RAY_BATCHES = (1, 2, 3, 4, 5, 6, 8, 10, 12, 14, 16, 20, 24, 32, 35, 64)


def stress_rays(lo, hi, seed: int = 7):
    """The stress test's incoherent rays: origins uniform in the scene box [lo, hi], directions
    uniform on the sphere, cut into the STRESS_RAY_BATCHES sizes. Returns (org, dir, sizes)."""
    sizes = [65536 * m for m in STRESS_RAY_BATCHES]
    org, d = random_rays(sum(sizes), lo, hi, seed)
    return org, d, sizes
