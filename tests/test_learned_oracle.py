"""CPU checks of the learned scorer's oracle pieces: the FP64 MLP against finite differences, the
realised-gain label against the SAH change of actually applying one reinsertion, the ordered
iteration against the plain chunked optimizer, and the feature definition."""
import numpy as np
import pytest

from bvhtest_gb300 import scenes
from oracle import mlp


def _params(seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    p = np.zeros(mlp.N_PARAMS)
    o = 0
    for name, shape in mlp.SIZES:
        n = int(np.prod(shape))
        fan = shape[1] if len(shape) == 2 else 64
        p[o:o + n] = rng.uniform(-1, 1, n) * np.sqrt(6.0 / fan) * scale
        o += n
    return p


def test_mlp_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(40, 24))
    t = rng.normal(size=40)
    p = _params(2)
    _, g = mlp.loss_and_grad(p, x, t, rounding=False)
    eps = 1e-6
    for i in rng.choice(mlp.N_PARAMS, 60, replace=False).tolist() + [mlp.N_PARAMS - 1]:
        d = np.zeros_like(p)
        d[i] = eps
        lp, _ = mlp.loss_and_grad(p + d, x, t, rounding=False)
        lm, _ = mlp.loss_and_grad(p - d, x, t, rounding=False)
        num = (lp - lm) / (2 * eps)
        assert abs(num - g[i]) <= 1e-6 + 1e-5 * abs(num), (i, num, g[i])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.1415926, 1e-30], np.float32)
    r = mlp.bf16_round(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie -> even
    assert r[2] == np.float32(1.0 + 4 * 2 ** -8)  # tie -> even (up)
    assert r[3] == -2.5
    assert abs(r[4] - 3.140625) < 1e-7
    assert np.array_equal(mlp.from_bf16_bits(mlp.bf16_bits(v)), r)


def test_adamw_matches_closed_form_first_step():
    p = np.array([1.0, -2.0])
    g = np.array([0.1, -0.3])
    out, _, _ = mlp.adamw_step(p, g, np.zeros(2), np.zeros(2), 1, 1e-3, 0.0)
    # the first Adam step moves every parameter by lr * sign(g) (up to eps)
    assert np.allclose(out, p - 1e-3 * np.sign(g), atol=1e-9)


def test_gain_equals_sah_change_of_applying_one_reinsertion(orc):
    vert, faces = scenes.uniform_soup(3000, seed=11)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    nodes = np.ascontiguousarray(nodes)
    feat, inner = orc.lr_features(nodes)
    gain, ok = orc.bn13_gains(nodes, inner)
    assert ok.mean() > 0.99
    s0 = orc.sah(nodes)
    pick = np.concatenate([np.argsort(-gain)[:6], np.argsort(gain)[:3], np.arange(5)])
    for i in pick.tolist():
        nd = nodes.copy()
        st = orc.bittner_iteration_ordered(nd, inner[i:i + 1], num_chunks=1, batch_percent=75.0)
        assert st["applied"] == int(ok[i])
        # the SAH with cInner = cLeaf = 1 changes by exactly the inner-node area change / root area
        assert abs((s0 - orc.sah(nd)) - gain[i]) <= 1e-6 * max(1.0, abs(gain[i])), (i, gain[i], s0 - orc.sah(nd))
        assert orc.validate(nd, vert, faces)[:4] == [0, 0, 0, 0]


def test_ordered_iteration_reproduces_the_plain_selection(orc):
    vert, faces = scenes.uniform_soup(5000, seed=12)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    ref, _, st_ref = orc.bittner_chunked(nodes, 1)
    # the plain order: stable descending inefficiency over the ascending inner-node list
    inner = np.nonzero(nodes["isLeafFlag"] == 0)[0].astype(np.uint32)
    cost = np.array([orc.lib().orc_inefficiency(orc._p(np.ascontiguousarray(nodes)), int(x)) for x in inner],
                    np.float32)
    order = inner[np.argsort(-cost, kind="stable")]
    nd = np.ascontiguousarray(nodes.copy())
    st = orc.bittner_iteration_ordered(nd, order)
    assert np.array_equal(nd.view(np.uint8), ref.view(np.uint8))
    assert st["applied"] == st_ref["applied"]


def test_feature_rows_follow_their_definition(orc):
    vert, faces = scenes.uniform_soup(2000, seed=13)
    nodes, _, _ = orc.lbvh_build(vert, faces)
    feat, inner = orc.lr_features(nodes)
    assert feat.shape == (1999, 24) and np.array_equal(inner, np.arange(1999))
    sa = nodes["surfaceArea"]
    root = feat[0]
    assert root[0] == np.float32(np.log2(sa[0])) and root[1] == 1.0 and root[2] == 1.0 and root[4] == 0.0
    assert root[5] + 0 >= 0 and 2 ** root[5] + 2 ** root[6] == pytest.approx(2000)
    x = 17
    l, r, p = nodes["left"][x], nodes["right"][x], nodes["parent"][x]
    assert feat[x, 1] == np.float32(sa[x] / sa[p])
    assert feat[x, 3] == np.float32(sa[x] / np.float32(sa[l] + sa[r]))
    assert np.all(feat[:, 14:] == 0)
    ranks = feat[:, 10:14]
    assert np.all((ranks >= 0) & (ranks <= 1))
    # the rank of the largest area is near 1, of the root's inefficiency between 0 and 1
    assert ranks[np.argmax(sa[:1999]), 3] > 0.99
    assert np.all(np.abs(feat[:, :10]) <= 64)
