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
