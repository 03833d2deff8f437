"""GPU checks of the learned reinsertion scorer against the oracle.

Features: bit-exact BF16 rows except the columns that go through log2f (at most one BF16 step
apart). Realised gains and training targets: bit-exact float32. MLP forward and gradient: FP32
accumulation against the FP64 restatement (oracle/mlp.py) with the same BF16 rounding points.
Learned selection: the GPU's order is the stable descending order of its own scores, and one
iteration driven by that order gives the oracle's tree byte for byte. Finally the trained scorer
must beat the plain inefficiency measure on held-out scenes.
"""
import numpy as np
import pytest

from bvhtest_gb300 import learned, scenes
from oracle import mlp

pytestmark = pytest.mark.gpu
LOG_COLS = [0, 5, 6, 7, 8, 9]  # features computed with log2f


def _tree(gpu, n, seed, topo="refCompat", iters=0):
    import torch
    v, f, nodes = learned.uniform_scene_tree(n, seed, topology=topo)
    if iters:
        opt = gpu.Bittner13GPU(nodes)
        opt.run(iters)
        torch.cuda.synchronize()
        opt.close()
    return v, f, nodes


def _bf16_to_f32(x):
    import torch
    return x.view(torch.int16).cpu().numpy().view(np.uint16).astype(np.uint32).__lshift__(16).view(np.float32)


@pytest.mark.parametrize("topo,iters", [("refCompat", 0), ("karras", 6)])
def test_features_match_oracle(gpu, orc, topo, iters):
    _, _, nodes = _tree(gpu, 20000, seed=31, topo=topo, iters=iters)
    host = gpu.nodes_to_numpy(nodes)
    ref, inner_ref = orc.lr_features(host)
    opt = gpu.Bittner13GPU(nodes)
    inner = opt.inner_nodes()
    assert np.array_equal(inner.cpu().numpy().view(np.uint32), inner_ref)
    x = _bf16_to_f32(gpu.LrFeatures(nodes.shape[0])(nodes, inner))
    r = mlp.bf16_round(ref)
    exact_cols = [c for c in range(24) if c not in LOG_COLS]
    assert np.array_equal(x[:, exact_cols], r[:, exact_cols])
    lx, lr_ = x[:, LOG_COLS], r[:, LOG_COLS]
    same = lx == lr_
    assert same.mean() > 0.999
    ulp = np.abs(lr_) * 2.0 ** -7
    assert np.all(np.abs(lx - lr_) <= ulp + 1e-30)


@pytest.mark.parametrize("topo,iters", [("refCompat", 0), ("refCompat", 8), ("karras", 3)])
def test_gains_match_oracle_bit_exact(gpu, orc, topo, iters):
    _, _, nodes = _tree(gpu, 12000, seed=32, topo=topo, iters=iters)
    host = gpu.nodes_to_numpy(nodes)
    opt = gpu.Bittner13GPU(nodes)
    inner = opt.inner_nodes()
    gain, tgt = opt.gains(inner, with_target=True)
    ref, ok = orc.bn13_gains(host, inner.cpu().numpy().view(np.uint32))
    g = gain.cpu().numpy()
    assert np.array_equal(g, ref), f"{np.count_nonzero(g != ref)} gains differ"
    assert ok.mean() > 0.99 and (ref > 0).mean() > 0.3
    leaves = host.shape[0] - inner.shape[0]
    want = np.sign(ref) * np.log1p(np.abs(ref).astype(np.float64) * np.float32(leaves / 0.16))
    assert np.allclose(tgt.cpu().numpy(), want, rtol=2e-6, atol=1e-7)
    # the tree is not modified by the evaluation
    assert np.array_equal(gpu.nodes_to_numpy(nodes).view(np.uint8), host.view(np.uint8))


def _rand_rows(n, seed):
    import torch
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1.5, (n, 24)).astype(np.float32)
    x[:, 14:] = 0
    xb = mlp.bf16_bits(x)
    xt = torch.from_numpy(xb.view(np.int16)).cuda().view(torch.bfloat16)
    return mlp.from_bf16_bits(xb), xt


def test_mlp_forward_matches_fp64(gpu):
    m = gpu.Mlp(seed=5)
    p = m.params()
    xf, xt = _rand_rows(20000, 1)
    y = m.forward(xt).cpu().numpy()
    ref, _ = mlp.forward(p, xf)
    err = np.abs(y - ref)
    assert np.quantile(err, 0.999) <= 1e-4 * (1 + np.abs(ref).max())
    assert err.max() <= 2e-2 * (1 + np.abs(ref).max())


def test_mlp_gradient_matches_fp64(gpu):
    import torch
    m = gpu.Mlp(seed=6)
    p = m.params()
    xf, xt = _rand_rows(5000, 2)
    t = np.tanh(xf[:, 0]) + 0.5 * xf[:, 1] * xf[:, 2]
    g, loss = m.gradient(xt, torch.from_numpy(t.astype(np.float32)).cuda())
    lref, gref = mlp.loss_and_grad(p, xf, t)
    assert abs(loss - lref) <= 1e-4 * lref
    assert np.linalg.norm(g - gref) <= 2e-3 * np.linalg.norm(gref)
    assert np.all(g[mlp.unpack(np.arange(mlp.N_PARAMS))["W1"][:, 14:].astype(int).ravel()] == 0)


def test_adamw_step_and_batch_rows_match_reference(gpu):
    import torch
    m = gpu.Mlp(seed=7)
    p0 = m.params().astype(np.float64)
    xf, xt = _rand_rows(3000, 3)
    t = (np.sin(xf[:, 0]) + xf[:, 3]).astype(np.float32)
    tt = torch.from_numpy(t).cuda()
    batch, seed, lr, wd = 512, 99, 1e-3, 1e-2
    rows = mlp.batch_rows(seed, 1, batch, 3000)
    g, loss_b = m.gradient(xt[torch.from_numpy(rows).cuda()], tt[torch.from_numpy(rows).cuda()])
    hist = m.train(xt, tt, 1, batch=batch, lr=lr, weight_decay=wd, seed=seed)
    lref, _ = mlp.loss_and_grad(p0, xf[rows], t[rows])
    assert abs(hist[0] - lref) <= 1e-4 * lref  # the step used exactly these rows
    p1, _, _ = mlp.adamw_step(p0, g.astype(np.float64), np.zeros(mlp.N_PARAMS), np.zeros(mlp.N_PARAMS), 1, lr, wd)
    assert np.allclose(m.params(), p1, rtol=1e-5, atol=1e-7)


def test_training_reduces_loss(gpu):
    import torch
    m = gpu.Mlp(seed=8)
    xf, xt = _rand_rows(50000, 4)
    t = torch.from_numpy((np.tanh(xf[:, 0]) + 0.5 * xf[:, 1] * xf[:, 2]).astype(np.float32)).cuda()
    hist = m.train(xt, t, 600, batch=2048, lr=3e-3, weight_decay=1e-4, seed=1)
    assert np.all(np.isfinite(hist))
    assert hist[-50:].mean() < 0.2 * hist[:10].mean()


def test_training_repeats_bit_for_bit(gpu):
    """The tiles' gradients are summed in a fixed order: the same data, initial weights and seed give
    the same weights, so a scorer trained in a run is the same scorer every run."""
    import torch
    xf, xt = _rand_rows(20000, 6)
    t = torch.from_numpy((np.tanh(xf[:, 0]) - 0.3 * xf[:, 3]).astype(np.float32)).cuda()
    got = []
    for _ in range(2):
        m = gpu.Mlp(seed=12)
        m.train(xt, t, 200, batch=4096, lr=2e-3, weight_decay=1e-4, seed=5)
        got.append(m.params())
    assert np.array_equal(got[0].view(np.uint32), got[1].view(np.uint32))


def test_learned_selection_iteration_matches_oracle(gpu, orc):
    import torch
    _, _, nodes = _tree(gpu, 16384, seed=33)
    start = gpu.nodes_to_numpy(nodes)
    m = gpu.Mlp(seed=9)
    opt = gpu.Bittner13GPU(nodes)
    opt.set_scorer(m)
    opt.select()
    order = opt.selection().cpu().numpy().view(np.uint32)
    # the order is the stable descending order of the scorer's own outputs
    inner = opt.inner_nodes()
    y = m.forward(gpu.LrFeatures(nodes.shape[0])(nodes, inner)).cpu().numpy()
    inn = inner.cpu().numpy().view(np.uint32)
    want = inn[np.argsort(-y, kind="stable")][: min(opt.batch_size, inn.shape[0])]
    assert np.array_equal(order, want)
    for c in range(32):
        opt.chunk(c)
    torch.cuda.synchronize()
    ref = np.ascontiguousarray(start.copy())
    orc.bittner_iteration_ordered(ref, order)
    assert np.array_equal(gpu.nodes_to_numpy(nodes).view(np.uint8), ref.view(np.uint8))
    # a full learned iteration through the graph path lands on the same tree as step()
    _, _, n2 = _tree(gpu, 16384, seed=33)
    o2 = gpu.Bittner13GPU(n2)
    o2.set_scorer(m)
    o2.run(2)
    _, _, n3 = _tree(gpu, 16384, seed=33)
    o3 = gpu.Bittner13GPU(n3)
    o3.set_scorer(m)
    o3.step()
    o3.step()
    torch.cuda.synchronize()
    assert torch.equal(n2, n3)


def test_trained_scorer_beats_the_plain_measure(gpu):
    """Train on pairs logged from plain runs over 6 scenes, evaluate on 2 unseen ones: the learned
    selection must reach the plain optimizer's 100-iteration SAH in at most 40 iterations, and after
    100 iterations of its own be at least 3% below it."""
    n = 16384
    trees = (_tree(gpu, n, seed=100 + s)[2] for s in range(6))
    data = learned.log_pairs(trees, iterations=60, every=3)
    assert data.x.shape[0] == 6 * 20 * (n - 1)
    m, hist, _ = learned.train(data, steps=3000, batch=8192, lr=1e-3)
    assert hist[-100:].mean() < 0.7 * hist[:20].mean()
    for seed in (7, 8):
        _, _, plain = _tree(gpu, n, seed)
        opt = gpu.Bittner13GPU(plain)
        opt.run(100)
        target = gpu.calc_sah(plain)
        _, _, lrn = _tree(gpu, n, seed)
        it, trace = learned.optimize_until(lrn, target, 100, scorer=m)
        assert it is not None and it <= 40, (seed, target, trace[::10])
        _, _, full = _tree(gpu, n, seed)
        lo = gpu.Bittner13GPU(full)
        lo.set_scorer(m)
        lo.run(100)
        assert gpu.calc_sah(full) < 0.97 * target


def test_policy_alternates_learned_and_plain_iterations(gpu):
    import torch
    _, _, nodes = _tree(gpu, 8192, seed=34)
    m = gpu.Mlp(seed=12)
    opt = gpu.Bittner13GPU(nodes)
    opt.set_scorer(m, 2)
    plain = gpu.Bittner13GPU(nodes)
    for it in range(4):
        assert opt.iteration == it
        opt.select()
        plain.select()
        same = torch.equal(opt.selection(), plain.selection())
        assert same == (it % 2 == 1), it  # odd iterations select by the inefficiency
        opt.step()
    opt.iteration = 0
    assert opt.iteration == 0
    opt.set_scorer(m, 0)  # scorer only
    opt.select()
    plain.select()
    assert not torch.equal(opt.selection(), plain.selection())
