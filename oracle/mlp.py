"""CPU restatement of the keypoint-credibility MLP (test infrastructure: the
checker of the GPU forward, backward and Adam kernels, never the product).

The network has no counterpart in the reference; it scores SHOT-352
keypoint descriptors so that low-credibility keypoints can be dropped before
matching.  Shape 352 -> 128 -> 64 -> 1 with ReLU, ReLU and a sigmoid
output.  Parameters, in this order (53,505 floats):

    W1[128][352], b1[128], W2[64][128], b2[64], w3[64], b3

The forward pass uses the weights rounded to bfloat16 (round to nearest
even); biases stay FP32.  The loss is the mean binary cross-entropy on the
logit z, written in its stable form max(z, 0) - y z + log1p(exp(-|z|)).
Gradients are taken with respect to the FP32 master weights (the rounding is
treated as the identity, the straight-through rule).  Adam (Kingma & Ba
2015) updates the FP32 master weights with bias-corrected moments.

Arithmetic here is FP64; the GPU accumulates in FP32, so the tests compare
within a relative tolerance.
"""
from __future__ import annotations

import numpy as np

D_IN, H1, H2 = 352, 128, 64
SIZES = [("W1", (H1, D_IN)), ("b1", (H1,)), ("W2", (H2, H1)), ("b2", (H2,)), ("w3", (H2,)), ("b3", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)  # 53,505


def unpack(theta: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = theta[o:o + n].reshape(shape)
        o += n
    return out


def pack(p: dict) -> np.ndarray:
    return np.concatenate([np.asarray(p[name], np.float64).ravel() for name, _ in SIZES])


def bf16_round(a) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even), returned as float32.
    NaN stays NaN (quieted)."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    r = r.astype(np.uint32)
    nan = np.isnan(a)
    r[nan] = (a.view(np.uint32)[nan] | 0x00400000) & 0xFFFF0000
    return r.view(np.float32)


def init_params(seed: int) -> np.ndarray:
    """He-uniform weights (bound sqrt(6 / fan_in)), zero biases, float32."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, shape in SIZES:
        if name.startswith("b"):
            p[name] = np.zeros(shape, np.float32)
        else:
            fan_in = shape[-1] if len(shape) == 2 else H2
            bound = np.sqrt(6.0 / fan_in)
            p[name] = rng.uniform(-bound, bound, shape).astype(np.float32)
    return pack(p).astype(np.float32)


def forward(theta: np.ndarray, X: np.ndarray):
    """Returns (h1, h2, z) in FP64 with bf16-rounded weights."""
    p = unpack(np.asarray(theta, np.float32))
    W1 = bf16_round(p["W1"]).astype(np.float64)
    W2 = bf16_round(p["W2"]).astype(np.float64)
    w3 = bf16_round(p["w3"]).astype(np.float64)
    X = np.asarray(X, np.float64)
    h1 = np.maximum(X @ W1.T + p["b1"].astype(np.float64), 0.0)
    h2 = np.maximum(h1 @ W2.T + p["b2"].astype(np.float64), 0.0)
    z = h2 @ w3 + float(p["b3"][0])
    return h1, h2, z


def score(theta: np.ndarray, X: np.ndarray) -> np.ndarray:
    return 1.0 / (1.0 + np.exp(-forward(theta, X)[2]))


def loss_and_grad(theta: np.ndarray, X: np.ndarray, y: np.ndarray):
    """Mean BCE loss and its gradient (FP64, length N_PARAMS)."""
    p = unpack(np.asarray(theta, np.float32))
    W2 = bf16_round(p["W2"]).astype(np.float64)
    w3 = bf16_round(p["w3"]).astype(np.float64)
    X = np.asarray(X, np.float64)
    y = np.asarray(y, np.float64)
    n = X.shape[0]
    h1, h2, z = forward(theta, X)
    loss = np.mean(np.maximum(z, 0.0) - y * z + np.log1p(np.exp(-np.abs(z))))
    dz = (1.0 / (1.0 + np.exp(-z)) - y) / n
    g = {"w3": h2.T @ dz, "b3": np.array([dz.sum()])}
    dh2 = np.outer(dz, w3) * (h2 > 0)
    g["W2"] = dh2.T @ h1
    g["b2"] = dh2.sum(0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    g["W1"] = dh1.T @ X
    g["b1"] = dh1.sum(0)
    return float(loss), pack(g)


def adam_step(theta, grad, m, v, t: int, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (t counts from 1).  Returns new (theta, m, v) in FP64."""
    theta = np.asarray(theta, np.float64)
    m = beta1 * np.asarray(m, np.float64) + (1 - beta1) * grad
    v = beta2 * np.asarray(v, np.float64) + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** t)
    vh = v / (1 - beta2 ** t)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v
