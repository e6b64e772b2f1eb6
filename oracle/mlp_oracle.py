"""Test infrastructure (the oracle), not product code.

NumPy restatement of the surrogate network's forward pass, loss and
backward pass, with BF16 rounding at the same points as the GPU kernels
(clode_gb300/csrc/host/mlp.cu): weights of the tensor-core layers, hidden
activations (the sine layer's sin and cos included) and the back-propagated
pre-activation gradients are rounded to BF16; products are accumulated in
float64 here (FP32 on the GPU), so the two agree to BF16 rounding of a few
ties, not bit for bit.

Network: h1 = sin(x W1 + b1), h2 = relu(h1 W2 + b2), h3 = relu(h2 W3 + b3),
out = h3 Wh + bh (H heads x K outputs).

Parameter vector layout (float32): W1 [2 x 256], b1 [256], W2 [256 x 256],
b2 [256], W3 [256 x 256], b3 [256], Wh [256 x H*K], bh [H*K].
"""
from __future__ import annotations

import numpy as np

WIDTH = 256


def _identity(a):
    return np.asarray(a, dtype=np.float64)


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


_bf16 = bf16


def split(params: np.ndarray, hk: int) -> dict:
    p = np.asarray(params, dtype=np.float64)
    sizes = [("W1", (2, WIDTH)), ("b1", (WIDTH,)), ("W2", (WIDTH, WIDTH)), ("b2", (WIDTH,)),
             ("W3", (WIDTH, WIDTH)), ("b3", (WIDTH,)), ("Wh", (WIDTH, hk)), ("bh", (hk,))]
    out, off = {}, 0
    for name, shape in sizes:
        n = int(np.prod(shape))
        out[name] = p[off:off + n].reshape(shape)
        off += n
    assert off == p.size, (off, p.size)
    return out


def forward(params: np.ndarray, x: np.ndarray, hk: int, exact: bool = False) -> dict:
    """`exact`: no BF16 rounding anywhere (float64 throughout), for checking
    the oracle's own gradients against finite differences."""
    bf16 = _identity if exact else _bf16
    P = split(params, hk)
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ P["W1"] + P["b1"]
    h1 = bf16(np.sin(z1))
    c1 = bf16(np.cos(z1))
    h2 = bf16(np.maximum(h1 @ bf16(P["W2"]) + P["b2"], 0.0))
    h3 = bf16(np.maximum(h2 @ bf16(P["W3"]) + P["b3"], 0.0))
    out = h3 @ bf16(P["Wh"]) + P["bh"]
    return {"P": P, "x": x, "h1": h1, "c1": c1, "h2": h2, "h3": h3, "out": out}


def loss_and_gradients(params: np.ndarray, x: np.ndarray, y: np.ndarray, heads: int, k: int,
                       exact: bool = False):
    bf16 = _identity if exact else _bf16
    hk = heads * k
    f = forward(params, x, hk, exact)
    P = f["P"]
    y_rep = np.tile(np.asarray(y, dtype=np.float64), (1, heads))
    d = f["out"] - y_rep
    loss = float(np.mean(d * d))
    dzo = bf16(2.0 * d / d.size)
    g = {}
    g["Wh"] = f["h3"].T @ dzo
    g["bh"] = dzo.sum(axis=0)
    dz3 = bf16((dzo @ bf16(P["Wh"]).T) * (f["h3"] > 0))
    g["W3"] = f["h2"].T @ dz3
    g["b3"] = dz3.sum(axis=0)
    dz2 = bf16((dz3 @ bf16(P["W3"]).T) * (f["h2"] > 0))
    g["W2"] = f["h1"].T @ dz2
    g["b2"] = dz2.sum(axis=0)
    dz1 = bf16((dz2 @ bf16(P["W2"]).T) * f["c1"])
    g["W1"] = f["x"].T @ dz1
    g["b1"] = dz1.sum(axis=0)
    flat = np.concatenate([g[n].ravel() for n in ("W1", "b1", "W2", "b2", "W3", "b3", "Wh", "bh")])
    return loss, flat, f
