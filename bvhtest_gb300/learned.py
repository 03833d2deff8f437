"""Learned reinsertion scorer: logging (feature row, realised SAH reduction) pairs from plain Bittner13
runs on the GPU, training the MLP with the library's own kernels, and optimising with it.

The reference has no learned part; this is the extension that replaces the inefficiency measure
(lib/builder/Bittner13CUDA.cu:480-500) by a prediction of the SAH a reinsertion actually removes.
Label of a node: the exact SAH reduction g (cInner = 1, in units of the root's surface area) of
removing it and reinserting its children alone against the current tree; training target:
sign(g) ln(1 + |g| numLeaves / 0.16), the gain in units of SA(root) / numLeaves, log-compressed so
that the nodes of every size are ranked on one scale; selection key: the prediction itself.
Everything runs on the device through libbvhgb; there is no CPU path.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import api, scenes


@dataclass
class TrainingSet:
    x: torch.Tensor  # [M, 24] bfloat16 feature rows (device)
    t: torch.Tensor  # [M] float32 targets (device)
    scenes: int = 0
    seconds: float = 0.0
    sah: list = field(default_factory=list)  # plain SAH trace per logged scene


def uniform_scene_tree(n: int, seed: int, morton_bits=30, topology="refCompat", builder: api.LBVH | None = None):
    """A uniform triangle soup (centroids in [0,1]^3, vertex offsets N(0, 0.004^2)) and its LBVH."""
    vert, faces = scenes.uniform_soup(n, seed=seed)
    v = torch.from_numpy(vert).cuda()
    f = torch.from_numpy(faces.view(np.int32)).cuda()
    b = builder or api.LBVH(n, morton_bits, topology)
    nodes = b.build(v, f)
    return v, f, nodes


def log_pairs(trees, iterations=100, every=4, batch_percent=1.0, num_chunks=32, with_sah=False, sample=1.0,
              seed=0) -> TrainingSet:
    """Run the plain optimizer on each node tensor of 'trees' for 'iterations' iterations; before every
    'every'-th iteration log the feature rows and realised-gain targets of all inner nodes, or of a
    random fraction 'sample' of them (drawn on the device from 'seed')."""
    xs, ts, sahs = [], [], []
    feats, feats_cap = None, 0
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    t0 = time.perf_counter()
    count = 0
    for nodes in trees:
        n = nodes.shape[0]
        if feats_cap < n:
            feats, feats_cap = api.LrFeatures(n), n
        opt = api.Bittner13GPU(nodes, batch_percent=batch_percent, num_chunks=num_chunks)
        inner = opt.inner_nodes()
        trace = []
        for it in range(iterations):
            if it % every == 0:
                x = feats(nodes, inner)
                cand = inner
                if sample < 1.0:
                    pick = torch.randperm(inner.shape[0], device="cuda", generator=gen)[: max(1, int(sample * inner.shape[0]))]
                    x, cand = x[pick], inner[pick]
                xs.append(x)
                _, tgt = opt.gains(cand, with_target=True)
                ts.append(tgt)
            if with_sah:
                trace.append(api.calc_sah(nodes))
            opt.step()
        if with_sah:
            trace.append(api.calc_sah(nodes))
            sahs.append(trace)
        opt.close()
        count += 1
    torch.cuda.synchronize()
    return TrainingSet(torch.cat(xs), torch.cat(ts), count, time.perf_counter() - t0, sahs)


def train(data: TrainingSet, steps=20000, batch=8192, lr=1e-3, weight_decay=1e-4, seed=0, init_seed=0):
    """A fresh scorer trained on 'data' by the library's kernels; returns (mlp, loss history, seconds)."""
    m = api.Mlp(seed=init_seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = m.train(data.x, data.t, steps, batch=batch, lr=lr, weight_decay=weight_decay, seed=seed)
    torch.cuda.synchronize()
    return m, hist, time.perf_counter() - t0


def optimize_until(nodes: torch.Tensor, target_sah: float, max_iterations: int, scorer: api.Mlp | None = None,
                   batch_percent=1.0, num_chunks=32):
    """Iterate (learned selection when a scorer is given) until the SAH is <= target_sah; returns
    (iterations, SAH trace). The SAH is read after every iteration, so this is for evaluation, not timing."""
    opt = api.Bittner13GPU(nodes, batch_percent=batch_percent, num_chunks=num_chunks)
    opt.set_scorer(scorer)
    trace = [api.calc_sah(nodes)]
    it = 0
    while it < max_iterations and trace[-1] > target_sah:
        opt.step()
        it += 1
        trace.append(api.calc_sah(nodes))
    opt.close()
    return (it if trace[-1] <= target_sah else None), trace


# ---- training families -----------------------------------------------------------------------

def uniform_family(n=65536, count=32, seed0=1000):
    """Config-4 training scenes: uniform soups of n triangles, 30-bit Morton, refCompat LBVH."""
    builder = api.LBVH(n, 30, "refCompat")
    for s in range(count):
        yield uniform_scene_tree(n, seed0 + s, builder=builder)[2].clone()


def large_family(n=262144, count=8, seed0=10, grid_cells=181):
    """Scenes of the large-scene generator at n triangles (a grid_cells^2 ground grid + a 64-component
    mixture), 63-bit Morton, karras LBVH."""
    b = api.LBVH(n, 63, "karras")
    for s in range(count):
        v_h, f_h = scenes.large_scene(n, seed=seed0 + s, grid_cells=grid_cells)
        yield b.build(torch.from_numpy(v_h).cuda(), torch.from_numpy(f_h.view(np.int32)).cuda())


FAMILIES = {
    "uniform": dict(trees=uniform_family, count=32, iterations=100, every=4),
    "large": dict(trees=large_family, count=8, iterations=200, every=8),
}


def train_family(name: str, steps=20000, batch=8192, lr=1e-3, weight_decay=1e-4, seed=0):
    """Log pairs from plain runs over the family's scenes and train a scorer; returns (mlp, info)."""
    f = FAMILIES[name]
    data = log_pairs(f["trees"](count=f["count"]), iterations=f["iterations"], every=f["every"])
    pairs, log_s = int(data.x.shape[0]), data.seconds
    m, hist, train_s = train(data, steps=steps, batch=batch, lr=lr, weight_decay=weight_decay, seed=seed)
    del data
    torch.cuda.empty_cache()
    return m, {"family": name, "scenes": f["count"], "pairs": pairs, "log_s": round(log_s, 2),
               "steps": steps, "batch": batch, "lr": lr, "weight_decay": weight_decay, "train_s": round(train_s, 2),
               "loss_first": round(float(hist[:100].mean()), 4), "loss_last": round(float(hist[-100:].mean()), 4)}


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(prog="python -m bvhtest_gb300.learned")
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train", help="log pairs from plain runs of a scene family and train a scorer")
    t.add_argument("--family", choices=sorted(FAMILIES), required=True)
    t.add_argument("--out", required=True, help="weights file (5825 little-endian float32)")
    t.add_argument("--steps", type=int, default=20000)
    a = ap.parse_args(argv)
    m, info = train_family(a.family, steps=a.steps)
    m.save(a.out)
    print(info, flush=True)


if __name__ == "__main__":
    main()
