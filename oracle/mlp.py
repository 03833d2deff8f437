"""FP64 restatement of the learned scorer's MLP (test infrastructure only; never used by the product).

The network is 24 -> 64 -> 64 -> 1 with GELU (tanh form of Hendrycks and Gimpel). As in the CUDA
kernels, inputs, weights and both hidden activations are BF16 values (round to nearest even from
FP32); everything else is computed here in float64. The backward treats each BF16 rounding as the
identity (straight-through), which is what the CUDA backward computes, and rounds the gradients of
both pre-activations to BF16, where the CUDA backward hands them to the tensor cores.

Parameter layout (5825 values): W1[64][24] b1[64] W2[64][64] b2[64] W3[64] b3[1].
"""
from __future__ import annotations

import numpy as np

N_IN, N_H = 24, 64
SIZES = [("W1", (N_H, N_IN)), ("b1", (N_H,)), ("W2", (N_H, N_H)), ("b2", (N_H,)), ("W3", (N_H,)), ("b3", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)
assert N_PARAMS == 5825
GELU_C = np.sqrt(2.0 / np.pi)
GELU_A = 0.044715


def bf16_round(x) -> np.ndarray:
    """Round to the nearest BF16 value (ties to even) through FP32; returns float32."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(f.shape)


def bf16_bits(x) -> np.ndarray:
    return (bf16_round(x).view(np.uint32) >> 16).astype(np.uint16)


def from_bf16_bits(b) -> np.ndarray:
    return (np.asarray(b, dtype=np.uint32) << 16).view(np.float32)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def pack(d) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SIZES])


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(GELU_C * (z + GELU_A * z ** 3)))


def gelu_grad(z):
    t = np.tanh(GELU_C * (z + GELU_A * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GELU_C * (1.0 + 3.0 * GELU_A * z * z)


def _round(v, rounding):
    return bf16_round(v).astype(np.float64) if rounding else v


def forward(params, x, rounding=True):
    """Returns (y, cache); params are the FP32 masters (rounded to BF16 here when rounding)."""
    P = unpack(_round(np.asarray(params, np.float64), rounding))
    x = _round(np.asarray(x, np.float64), rounding)
    z1 = x @ P["W1"].T + P["b1"]
    a1 = _round(gelu(z1), rounding)
    z2 = a1 @ P["W2"].T + P["b2"]
    a2 = _round(gelu(z2), rounding)
    y = a2 @ P["W3"] + P["b3"][0]
    return y, (P, x, z1, a1, z2, a2)


def loss_and_grad(params, x, t, rounding=True):
    """Mean squared error over all rows and its gradient (float64, layout of the parameters)."""
    y, (P, x, z1, a1, z2, a2) = forward(params, x, rounding)
    n = x.shape[0]
    d = y - np.asarray(t, np.float64)
    loss = float(np.sum(d * d) / n)
    dy = 2.0 * d / n
    g = {"W3": a2.T @ dy, "b3": np.array([dy.sum()])}
    # the CUDA backward feeds dz2 and dz1 to the tensor cores as BF16: they are rounded there
    dz2 = _round(np.outer(dy, P["W3"]) * gelu_grad(z2), rounding)
    g["W2"] = dz2.T @ a1
    g["b2"] = dz2.sum(0)
    dz1 = _round((dz2 @ P["W2"]) * gelu_grad(z1), rounding)
    g["W1"] = dz1.T @ x
    g["b1"] = dz1.sum(0)
    return loss, pack(g)


def is_bias(i: int) -> bool:
    o, spans = 0, []
    for name, shape in SIZES:
        n = int(np.prod(shape))
        spans.append((name, o, o + n))
        o += n
    return any(name.startswith("b") and a <= i < b for name, a, b in spans)


BIAS_MASK = np.array([is_bias(i) for i in range(N_PARAMS)])


def adamw_step(p, g, m, v, step, lr, wd, b1=0.9, b2=0.999, eps=1e-8):
    """One AdamW update (decoupled decay on weights only); step counts from 1. Returns (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    bias = BIAS_MASK if p.shape == BIAS_MASK.shape else np.zeros(p.shape, bool)
    p = np.where(bias, p, p - lr * wd * p)
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v


def batch_rows(seed: int, step: int, batch: int, num_samples: int) -> np.ndarray:
    """The rows of training step 'step' (from 1): SplitMix64 of seed + golden * (step * batch + i + 1)."""
    M = (1 << 64) - 1
    out = np.zeros(batch, np.int64)
    for i in range(batch):
        z = (seed + 0x9E3779B97F4A7C15 * (step * batch + i + 1)) & M
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        z ^= z >> 31
        out[i] = z % num_samples
    return out
