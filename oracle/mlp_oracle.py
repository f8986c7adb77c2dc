"""CPU oracle of the learned level scheduler's network (TEST INFRASTRUCTURE ONLY).

numpy restatement of the 4 -> 64 -> 64 -> 8 ReLU MLP with softmax cross-entropy
that nsphere_gb300/csrc/nsg_mlp.cu trains and runs on the GPU.  Two modes:

* ``exact``: float64 throughout -- used to check the analytic backward pass against
  finite differences;
* ``bf16``: rounds to bfloat16 exactly where the GPU kernels do (weights, inputs,
  hidden activations, the back-propagated errors fed to the tensor cores) and
  accumulates in float64, so the GPU's FP32-accumulated gradients must agree to
  accumulation-order differences.

Parameter vector layout (as in the library): W1[64][16] (inputs 4..15 zero), b1[64],
W2[64][64], b2[64], W3[8][64], b3[8].
"""
from __future__ import annotations

import numpy as np

H, IN, OUT = 64, 16, 8
SIZES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (OUT, H)), ("b3", (OUT,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(w):
    out, k = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(w[k:k + n], dtype=np.float64).reshape(shape)
        k += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SIZES])


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    x = np.asarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def forward_backward(w, X, y, cls_w, mode="exact"):
    """Summed weighted cross-entropy and its gradient (same layout as w)."""
    P = unpack(w)
    rnd = bf16 if mode == "bf16" else (lambda a: np.asarray(a, dtype=np.float64))
    f32 = (lambda a: np.asarray(a, dtype=np.float32).astype(np.float64)) if mode == "bf16" else rnd
    nb = X.shape[0]
    X16 = np.zeros((nb, IN))
    X16[:, :4] = X
    Xb = rnd(X16)
    W1, W2, W3 = rnd(P["W1"]), rnd(P["W2"]), rnd(P["W3"])
    b1, b2, b3 = f32(P["b1"]), f32(P["b2"]), f32(P["b3"])
    z1 = Xb @ W1.T + b1
    h1 = rnd(np.maximum(z1, 0.0))
    z2 = h1 @ W2.T + b2
    h2 = rnd(np.maximum(z2, 0.0))
    lg = h2 @ W3.T + b3
    lg = lg - lg.max(axis=1, keepdims=True)
    p = np.exp(lg)
    p /= p.sum(axis=1, keepdims=True)
    wts = np.asarray(cls_w, dtype=np.float64)[y]
    loss = float(np.sum(-wts * np.log(np.maximum(p[np.arange(nb), y], 1e-300))))
    dz3 = p.copy()
    dz3[np.arange(nb), y] -= 1.0
    dz3 *= wts[:, None]
    dz3b = rnd(dz3)
    g = {}
    g["b3"] = dz3.sum(axis=0)
    g["W3"] = dz3b.T @ h2
    dz2 = (dz3b @ W3) * (h2 > 0)
    g["b2"] = dz2.sum(axis=0)
    dz2b = rnd(dz2)
    g["W2"] = dz2b.T @ h1
    dz1 = (dz2b @ W2) * (h1 > 0)
    g["b1"] = dz1.sum(axis=0)
    dz1b = rnd(dz1)
    g["W1"] = dz1b.T @ Xb
    g["W1"][:, 4:] = 0.0
    return loss, pack(g)


def predict(w, X, mode="bf16"):
    P = unpack(w)
    rnd = bf16 if mode == "bf16" else (lambda a: np.asarray(a, dtype=np.float64))
    X16 = np.zeros((X.shape[0], IN))
    X16[:, :4] = X
    h1 = rnd(np.maximum(rnd(X16) @ rnd(P["W1"]).T + P["b1"], 0.0))
    h2 = rnd(np.maximum(h1 @ rnd(P["W2"]).T + P["b2"], 0.0))
    lg = h2 @ rnd(P["W3"]).T + P["b3"]
    return np.argmax(lg, axis=1), lg


def random_weights(seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    P = {}
    P["W1"] = np.zeros((H, IN))
    P["W1"][:, :4] = rng.uniform(-1, 1, (H, 4)) * np.sqrt(6 / 4) * scale
    P["b1"] = rng.uniform(-0.1, 0.1, H)
    P["W2"] = rng.uniform(-1, 1, (H, H)) * np.sqrt(6 / H) * scale
    P["b2"] = rng.uniform(-0.1, 0.1, H)
    P["W3"] = rng.uniform(-1, 1, (OUT, H)) * np.sqrt(6 / H) * scale
    P["b3"] = rng.uniform(-0.1, 0.1, OUT)
    return pack(P)
