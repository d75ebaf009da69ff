"""NumPy restatement of the learned refinement estimator (adaptivemesh_gb300/csrc/estimator.cu):
forward pass, mean-squared-error loss and its gradients, in float64 with the GPU's BF16 roundings
applied at the same points (the GEMM operands: im2col matrices, weights, activations and the
back-propagated gradients).

TEST INFRASTRUCTURE ONLY: what the GPU network's forward pass and gradients are compared with.  The
reference has no learned estimator; the network, its layouts and its parameter vector are this
library's (documented in include/amr_gb300.h, amr_estimator_get_params).
"""
from __future__ import annotations

import numpy as np

K1, K1R, K2, K3, C1, C2, F = 96, 81, 432, 1024, 16, 16, 32
SIZES = [("W1", (K1, C1)), ("b1", (C1,)), ("W2", (K2, C2)), ("b2", (C2,)), ("W3", (K3, F)), ("b3", (F,)),
         ("W4", (F,)), ("b4", (1,))]


EXACT = False   # set by the self-check: no BF16 rounding (the finite-difference test of the algebra)


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest, ties to even) and back, as float64."""
    if EXACT:
        return np.asarray(x, np.float64)
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(params[o:o + n], np.float64).reshape(shape)
        o += n
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], np.float64).reshape(-1) for name, _ in SIZES])


def _taps():
    return [(dz, dy, dx) for dz in range(3) for dy in range(3) for dx in range(3)]


def im2col1(x: np.ndarray) -> np.ndarray:
    """x [B][3][8][8][8] -> [B*512][96]: column c*27 + tap, zero padding, columns 81..95 zero."""
    B = x.shape[0]
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1), (1, 1)))
    cols = np.zeros((B, 8, 8, 8, K1))
    for c in range(3):
        for t, (dz, dy, dx) in enumerate(_taps()):
            cols[..., c * 27 + t] = xp[:, c, dz:dz + 8, dy:dy + 8, dx:dx + 8]
    return cols.reshape(B * 512, K1)


def im2col2(h1: np.ndarray) -> np.ndarray:
    """h1 [B][512][16] (position z-major, channel last) -> [B*64][432], stride 2, padding 1."""
    B = h1.shape[0]
    v = h1.reshape(B, 8, 8, 8, C1)
    vp = np.pad(v, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    cols = np.zeros((B, 4, 4, 4, K2))
    for c in range(C1):
        for t, (dz, dy, dx) in enumerate(_taps()):
            cols[..., c * 27 + t] = vp[:, dz:dz + 8:2, dy:dy + 8:2, dx:dx + 8:2, c]
    return cols.reshape(B * 64, K2)


def col2im2(da: np.ndarray, B: int) -> np.ndarray:
    """Adjoint of im2col2: [B*64][432] -> [B][512][16]."""
    d = da.reshape(B, 4, 4, 4, K2)
    out = np.zeros((B, 10, 10, 10, C1))
    for c in range(C1):
        for t, (dz, dy, dx) in enumerate(_taps()):
            out[:, dz:dz + 8:2, dy:dy + 8:2, dx:dx + 8:2, c] += d[..., c * 27 + t]
    return out[:, 1:9, 1:9, 1:9, :].reshape(B, 512, C1)


def forward(params: np.ndarray, x: np.ndarray) -> dict:
    """Forward pass of B tiles; returns every intermediate the backward pass needs."""
    p = unpack(params)
    B = x.shape[0]
    a1 = bf16(im2col1(x.reshape(B, 3, 8, 8, 8)))
    z1 = a1 @ bf16(p["W1"]) + p["b1"]
    h1 = bf16(np.maximum(z1, 0)).reshape(B, 512, C1)
    a2 = im2col2(h1)
    z2 = a2 @ bf16(p["W2"]) + p["b2"]
    h2 = bf16(np.maximum(z2, 0)).reshape(B, K3)
    z3 = h2 @ bf16(p["W3"]) + p["b3"]
    h3 = bf16(np.maximum(z3, 0))
    out = h3 @ bf16(p["W4"]) + p["b4"][0]
    return {"p": p, "a1": a1, "z1": z1, "h1": h1, "a2": a2, "z2": z2, "h2": h2, "z3": z3, "h3": h3, "out": out}


def gradients(params: np.ndarray, x: np.ndarray, t: np.ndarray) -> tuple[np.ndarray, float]:
    """Gradients of mean((out - t)^2) with respect to the parameter vector, and the loss."""
    f = forward(params, x)
    p = f["p"]
    B = x.shape[0]
    d = f["out"] - t
    loss = float(np.mean(d * d))
    dout = 2 * d / B
    g = {}
    g["W4"] = f["h3"].T @ dout
    g["b4"] = np.array([dout.sum()])
    dh3 = dout[:, None] * bf16(p["W4"])[None, :]
    dz3 = np.where(f["z3"] > 0, dh3, 0.0)
    g["b3"] = dz3.sum(0)
    dz3b = bf16(dz3)
    g["W3"] = f["h2"].T @ dz3b
    dh2 = dz3b @ bf16(p["W3"]).T
    dz2 = np.where(f["z2"].reshape(B, K3) > 0, dh2, 0.0).reshape(B * 64, C2)
    g["b2"] = dz2.sum(0)
    dz2b = bf16(dz2)
    g["W2"] = f["a2"].T @ dz2b
    da2 = dz2b @ bf16(p["W2"]).T
    dh1 = col2im2(da2, B).reshape(B * 512, C1)
    dz1 = np.where(f["z1"] > 0, dh1, 0.0)
    g["b1"] = dz1.sum(0)
    g["W1"] = f["a1"].T @ bf16(dz1)
    return pack(g), loss
