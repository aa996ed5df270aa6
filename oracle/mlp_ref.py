"""FP64 reference of the learned control variate's network -- TEST INFRASTRUCTURE (the checker of the
device forward/backward kernels), not the product.

The network (viltrum_gb300/csrc/k_mlp.cuh): input u in [0,1]^D (the point mapped into the range),
features [u_d, sin(2^k pi u_d), cos(2^k pi u_d) for k < 6] (13 D values, zero-padded to FIN, a multiple
of 16), four hidden layers of width 64 with ReLU, and a linear output.  Weights are BF16 on the
device, accumulation FP32; activations are rounded to BF16 where the device feeds them to the tensor
cores.  This reference rounds at exactly the same points (round-to-nearest-even BF16) and computes
everything else in FP64, so device results agree with it to FP32 accumulation error.

Parameter layout (flat float32): W0[FIN,64], b0[64], W1[64,64], b1, W2[64,64], b2, W3[64,64], b3,
w4[64], b4[1].
"""
from __future__ import annotations

import numpy as np

WIDTH = 64
BANDS = 6


def fin(dim: int) -> int:
    return ((13 * dim + 15) // 16) * 16


def n_params(dim: int) -> int:
    f = fin(dim)
    return f * WIDTH + WIDTH + 3 * (WIDTH * WIDTH + WIDTH) + WIDTH + 1


def bf16(a):
    """round float64/float32 values to bfloat16 (nearest even), returned as float64"""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = rounded.astype(np.uint32).view(np.float32).astype(np.float64)
    return np.where(np.isnan(a), np.nan, out)


def unpack(theta: np.ndarray, dim: int):
    f = fin(dim)
    p = np.asarray(theta, dtype=np.float64)
    o = 0
    out = []
    for (a, b) in [(f, WIDTH), (WIDTH, WIDTH), (WIDTH, WIDTH), (WIDTH, WIDTH)]:
        W = p[o:o + a * b].reshape(a, b)
        o += a * b
        bias = p[o:o + b]
        o += b
        out.append((W, bias))
    w4 = p[o:o + WIDTH]
    o += WIDTH
    b4 = p[o]
    return out, w4, b4


def features(u: np.ndarray) -> np.ndarray:
    n, dim = u.shape
    cols = [u[:, d] for d in range(dim)]
    for d in range(dim):
        for k in range(BANDS):
            a = (2.0 ** k) * u[:, d]
            cols.append(np.sin(np.pi * a))
            cols.append(np.cos(np.pi * a))
    F = np.zeros((n, fin(dim)))
    F[:, :len(cols)] = np.stack(cols, axis=1)
    return F


def init(dim: int, seed: int) -> np.ndarray:
    """He-uniform initial weights, zero biases (SplitMix64-seeded numpy generator)."""
    rng = np.random.default_rng(seed)
    parts = []
    f = fin(dim)
    for a, b in [(f, WIDTH), (WIDTH, WIDTH), (WIDTH, WIDTH), (WIDTH, WIDTH)]:
        lim = np.sqrt(6.0 / a)
        parts.append(rng.uniform(-lim, lim, size=a * b))
        parts.append(np.zeros(b))
    parts.append(rng.uniform(-np.sqrt(6.0 / WIDTH), np.sqrt(6.0 / WIDTH), size=WIDTH))
    parts.append(np.zeros(1))
    return np.concatenate(parts).astype(np.float32)


def forward_backward(theta: np.ndarray, u: np.ndarray, y: np.ndarray | None = None, feat_fn=None):
    """Outputs and (if y is given) the gradient of mean((g-y)^2) with the device's BF16 roundings."""
    dim = u.shape[1]
    layers, w4, b4 = unpack(theta, dim)
    F = features(u) if feat_fn is None else feat_fn(u)
    acts = [bf16(F)]                      # tensor-core inputs are BF16
    masks = []
    for W, b in layers:
        z = acts[-1] @ bf16(W) + b        # FP32 accumulation of BF16 products, + FP32 bias
        h = np.maximum(z, 0.0)
        masks.append(z > 0)
        acts.append(bf16(h))
    out = acts[-1] @ w4 + b4              # FP32 output layer on the BF16 activations
    if y is None:
        return out, None
    n = u.shape[0]
    dout = 2.0 * (out - y) / n
    grads = [None] * 4
    g_w4 = acts[-1].T @ dout
    g_b4 = dout.sum()
    dz = bf16(np.outer(dout, w4) * masks[3])        # dZ is a tensor-core operand: BF16
    for l in range(3, -1, -1):
        W, _ = layers[l]
        gW = acts[l].T @ dz
        gb = dz.sum(axis=0)
        grads[l] = (gW, gb)
        if l > 0:
            dh = dz @ bf16(W).T
            dz = bf16(dh * masks[l - 1])
    flat = []
    for gW, gb in grads:
        flat.append(gW.ravel())
        flat.append(gb)
    flat.append(g_w4)
    flat.append(np.array([g_b4]))
    return out, np.concatenate(flat)
