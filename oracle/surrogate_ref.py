"""FP64 CPU reference of the sky-map surrogate's forward and backward pass -- TEST INFRASTRUCTURE
ONLY (the checker of csrc/exc_mlp.cu's training kernels; only tests/ import it).

The network (surrogate/model.py): Fourier features x0 [B, 256] -> depth x (Linear 256 -> 256,
SiLU) -> Linear head 256 -> n_out; loss = sum over rows and outputs of (y - t)^2, whose mean
over the B * n_out terms is what training minimises (dL/dy = 2 (y - t) / (B n_out)).

`forward_backward` evaluates it in float64 with numpy. With `bf16=True` it rounds to bfloat16
exactly where the kernels store bfloat16: each layer's pre-activation Z and activation H (the
SiLU of the rounded Z), and each layer's back-propagated gradient dZ (after the SiLU
derivative, taken at the rounded Z). Everything else -- the GEMM sums, the bias and head
terms, the loss and the weight and bias gradients -- is exact float64 arithmetic. The kernels
differ from it only by their float32 accumulation (about 1e-6 relative per sum) and by the
rare bfloat16 rounding that this moves across a rounding midpoint; with `bf16=False` it is the
network's exact-arithmetic gradient, from which bfloat16 storage alone departs by about
2^-8 relative.
"""
from __future__ import annotations

import numpy as np


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round float64 values to the nearest bfloat16 (ties to even), via float32 as the kernels'
    float32 values are rounded (the float64 -> float32 step is exact for float32 inputs)."""
    f = np.asarray(x, dtype=np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> np.uint64(16)) & np.uint64(1)
    r = ((u + np.uint64(0x7FFF) + lsb) >> np.uint64(16)) << np.uint64(16)
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    return np.where(np.isfinite(f), out, f.astype(np.float64))


def _sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * _sigmoid(z)


def dsilu(z):
    s = _sigmoid(z)
    return s * (1.0 + z * (1.0 - s))


def forward_backward(x0, W, b, Wh, bh, t, bf16: bool = True) -> dict:
    """One member: x0 [B, 256] (the features), W [depth][256, 256] and b [depth][256] (layer
    l maps its input h to h W[l]^T + b[l]), Wh [n_out, 256], bh [n_out], targets t [B, n_out].
    Returns {"loss": sum (y - t)^2, "y": y, "gw": [...], "gb": [...], "gwh", "gbh"}."""
    rnd = bf16_round if bf16 else (lambda v: v)
    x0 = np.asarray(x0, dtype=np.float64)
    B = x0.shape[0]
    n_out = Wh.shape[0]
    h = x0
    Z, H = [], [x0]
    for Wl, bl in zip(W, b):
        z = rnd(h @ np.asarray(Wl, np.float64).T + np.asarray(bl, np.float64))
        h = rnd(silu(z))
        Z.append(z)
        H.append(h)
    y = h @ np.asarray(Wh, np.float64).T + np.asarray(bh, np.float64)
    d = y - np.asarray(t, np.float64)
    dy = 2.0 * d / (B * n_out)
    out = {"loss": float(np.sum(d * d)), "y": y, "gwh": dy.T @ h, "gbh": dy.sum(0)}
    dz = rnd((dy @ np.asarray(Wh, np.float64)) * dsilu(Z[-1]))
    gw, gb = [None] * len(W), [None] * len(W)
    for l in range(len(W) - 1, -1, -1):
        gw[l] = dz.T @ H[l]
        gb[l] = dz.sum(0)
        if l > 0:
            dz = rnd((dz @ np.asarray(W[l], np.float64)) * dsilu(Z[l - 1]))
    out["gw"], out["gb"] = gw, gb
    return out


def features(uv: np.ndarray, n_freq: int) -> np.ndarray:
    """The Fourier features in float64: [sin(pi k u), cos(pi k u), sin(pi k v), cos(pi k v)] for
    k = 1..n_freq, u and v the tangent-plane coordinates (already centred and scaled)."""
    uv = np.asarray(uv, dtype=np.float64)
    k = np.arange(1, n_freq + 1, dtype=np.float64)
    pu, pv = np.pi * uv[:, :1] * k, np.pi * uv[:, 1:2] * k
    return np.concatenate([np.sin(pu), np.cos(pu), np.sin(pv), np.cos(pv)], axis=1)
