"""CPU restatement of the learned-solve network (test infrastructure, not shipped).

The network has no counterpart in the reference: this numpy FP64 version of its
forward pass, loss and gradient is the check for the GPU training kernels (gradient
check) and, with BF16 rounding of weights, inputs and hidden activations, for the
tensor-core inference kernel.

Blob layout (FP32): feature mean[16], feature std[16], W1[64][16], b1[64], W2[64][64],
b2[64], W3[64][64], b3[64], W4[2][64], b4[2].  Sample: features[16], y, g.
Loss per sample: (out0 - y)^2 + (y - (1 + 0.25 tanh(out1)) g)^2, averaged over samples.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

OFF = {}
_o = 0
for _name, _size in (("mu", 16), ("sd", 16), ("W1", 64 * 16), ("b1", 64), ("W2", 64 * 64), ("b2", 64),
                     ("W3", 64 * 64), ("b3", 64), ("W4", 2 * 64), ("b4", 2)):
    OFF[_name] = (_o, _size)
    _o += _size
BLOB_FLOATS = _o
SHAPES = {"W1": (64, 16), "W2": (64, 64), "W3": (64, 64), "W4": (2, 64)}
SCALE_RANGE = 0.25


def unpack(blob):
    out = {}
    for k, (o, n) in OFF.items():
        a = np.asarray(blob[o:o + n], dtype=np.float64)
        out[k] = a.reshape(SHAPES[k]) if k in SHAPES else a
    return out


def pack(parts) -> np.ndarray:
    blob = np.zeros(BLOB_FLOATS, dtype=np.float32)
    for k, (o, n) in OFF.items():
        blob[o:o + n] = np.asarray(parts[k], dtype=np.float32).ravel()
    return blob


def init_blob(mu, sd, seed=0) -> np.ndarray:
    """He-style initialisation (seeded), zero biases, small output layer."""
    rng = np.random.default_rng(seed)
    p = {"mu": mu, "sd": sd}
    for k, (fo, fi) in SHAPES.items():
        scale = np.sqrt(2.0 / fi) * (0.1 if k == "W4" else 1.0)
        p[k] = rng.standard_normal((fo, fi)) * scale
    for k in ("b1", "b2", "b3"):
        p[k] = np.zeros(64)
    p["b4"] = np.zeros(2)
    return pack(p)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def bf16(a):
    """Round to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(blob, feats, bf16_path=False):
    """Network outputs (n, 2) for (n, 16) features (residual features already scaled)."""
    P = unpack(blob)
    x = (np.asarray(feats, dtype=np.float64) - P["mu"]) / P["sd"]
    if bf16_path:
        x = bf16(x)
    h = x
    for k in ("1", "2", "3"):
        W = bf16(P["W" + k]) if bf16_path else P["W" + k]
        z = h @ W.T + P["b" + k]
        h = gelu(z)
        if bf16_path:
            h = bf16(h)
    W4 = bf16(P["W4"]) if bf16_path else P["W4"]
    return h @ W4.T + P["b4"]


def loss_grad(blob, samples):
    """Mean loss and its gradient (blob layout; mean/std entries zero), FP64."""
    P = unpack(blob)
    s = np.asarray(samples, dtype=np.float64)
    n = s.shape[0]
    x = (s[:, :16] - P["mu"]) / P["sd"]
    y, g = s[:, 16], s[:, 17]
    z1 = x @ P["W1"].T + P["b1"]; a1 = gelu(z1)
    z2 = a1 @ P["W2"].T + P["b2"]; a2 = gelu(z2)
    z3 = a2 @ P["W3"].T + P["b3"]; a3 = gelu(z3)
    o = a3 @ P["W4"].T + P["b4"]
    th = np.tanh(o[:, 1])
    r0 = o[:, 0] - y
    r1 = y - (1.0 + SCALE_RANGE * th) * g
    loss = np.mean(r0 * r0 + r1 * r1)
    d4 = np.stack([2.0 * r0, -2.0 * r1 * g * SCALE_RANGE * (1.0 - th * th)], axis=1) / n
    G = {"W4": d4.T @ a3, "b4": d4.sum(0)}
    d3 = (d4 @ P["W4"]) * gelu_grad(z3)
    G["W3"] = d3.T @ a2; G["b3"] = d3.sum(0)
    d2 = (d3 @ P["W3"]) * gelu_grad(z2)
    G["W2"] = d2.T @ a1; G["b2"] = d2.sum(0)
    d1 = (d2 @ P["W2"]) * gelu_grad(z1)
    G["W1"] = d1.T @ x; G["b1"] = d1.sum(0)
    G["mu"] = np.zeros(16); G["sd"] = np.zeros(16)
    grad = np.zeros(BLOB_FLOATS)
    for k, (o_, m) in OFF.items():
        grad[o_:o_ + m] = np.asarray(G[k]).ravel()
    return loss, grad
