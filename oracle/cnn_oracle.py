"""FP64 numpy oracle of the subgrid-closure CNN (test infrastructure only).

Architecture (the learned-closure form; no counterpart in the reference):
6 convolutions 3x3 with circular padding, 2 -> 32 -> 32 -> 32 -> 32 -> 32 -> 1
channels, GELU (erf form) after the first five, mean-squared-error loss.
Tensors are NHWC; a conv weight is ``W[co, tap, ci]`` with tap = 3*(dy+1)+(dx+1)
and ``out[p] = b + sum_tap W[:, tap, :] @ in[p + (dy, dx)]`` (periodic).

``bf16`` rounds to bfloat16 (round to nearest even) so the oracle can be fed
the same quantised weights and inputs as the GPU kernels.
"""

from __future__ import annotations

import math

import numpy as np

CHANNELS = [2, 32, 32, 32, 32, 32, 1]
TAPS = [(dy, dx) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float values to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + np.vectorize(math.erf)(x / math.sqrt(2.0)))


def gelu_grad(x):
    cdf = 0.5 * (1.0 + np.vectorize(math.erf)(x / math.sqrt(2.0)))
    pdf = np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)
    return cdf + x * pdf


def shift(x: np.ndarray, dy: int, dx: int) -> np.ndarray:
    """y[b, i, j] = x[b, (i+dy) mod H, (j+dx) mod W]."""
    return np.roll(np.roll(x, -dy, axis=1), -dx, axis=2)


def conv(x: np.ndarray, W: np.ndarray, b: np.ndarray) -> np.ndarray:
    out = np.zeros(x.shape[:3] + (W.shape[0],))
    for t, (dy, dx) in enumerate(TAPS):
        out += shift(x, dy, dx) @ W[:, t, :].T
    return out + b


def forward(params, x):
    """params: list of (W, b); x: (B, H, W, 2).  Returns (y, cache)."""
    acts, pres = [x], []
    h = x
    for i, (W, b) in enumerate(params):
        z = conv(h, W, b)
        pres.append(z)
        h = gelu(z) if i < len(params) - 1 else z
        acts.append(h)
    return h[..., 0], (acts, pres)


def loss_and_grads(params, x, target):
    """MSE over every output pixel; returns (loss, [(dW, db)], dx)."""
    y, (acts, pres) = forward(params, x)
    n = y.size
    loss = float(np.mean((y - target) ** 2))
    dz = np.zeros_like(pres[-1])
    dz[..., 0] = 2.0 * (y - target) / n
    grads = [None] * len(params)
    for i in range(len(params) - 1, -1, -1):
        W, b = params[i]
        a_in = acts[i]
        dW = np.zeros_like(W)
        for t, (dy, dx) in enumerate(TAPS):
            sh = shift(a_in, dy, dx)
            dW[:, t, :] = np.einsum("bhwo,bhwi->oi", dz, sh)
        db = dz.sum(axis=(0, 1, 2))
        grads[i] = (dW, db)
        da = np.zeros_like(a_in)
        for t, (dy, dx) in enumerate(TAPS):
            da += shift(dz @ W[:, t, :], -dy, -dx)
        if i > 0:
            dz = da * gelu_grad(pres[i - 1])
        else:
            dx_in = da
    return loss, grads, dx_in
