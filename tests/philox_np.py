"""Philox4x32-10 in numpy (Salmon et al., SC'11), used by the tests to reproduce the exact sample
points the device draws for sample j of bin b: counter (j, b_lo, b_hi, block), key = seed."""
import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    c0, c1, c2, c3 = (np.asarray(c, dtype=np.uint32) for c in (c0, c1, c2, c3))
    k0 = np.uint32(k0)
    k1 = np.uint32(k1)
    with np.errstate(over="ignore"):
        for _ in range(10):
            p0 = M0 * c0.astype(np.uint64)
            p1 = M1 * c2.astype(np.uint64)
            hi0, lo0 = (p0 >> np.uint64(32)).astype(np.uint32), (p0 & MASK).astype(np.uint32)
            hi1, lo1 = (p1 >> np.uint64(32)).astype(np.uint32), (p1 & MASK).astype(np.uint32)
            c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
            k0 = np.uint32(k0 + W0)
            k1 = np.uint32(k1 + W1)
    return c0, c1, c2, c3


def u01(r):
    return (np.asarray(r, np.uint32) >> np.uint32(8)).astype(np.float32) * np.float32(5.9604644775390625e-08)


def points(bin_index: int, spp: int, dim: int, seed: int, lo, w):
    """sample points of one bin exactly as the device computes them (u*w + lo in float32)"""
    j = np.arange(spp, dtype=np.uint32)
    out = np.empty((spp, dim), np.float32)
    for blk in range((dim + 3) // 4):
        r = philox4x32_10(j, np.full(spp, bin_index & 0xFFFFFFFF, np.uint32), np.full(spp, bin_index >> 32, np.uint32),
                          np.full(spp, blk, np.uint32), seed & 0xFFFFFFFF, seed >> 32)
        for k in range(4):
            d = 4 * blk + k
            if d < dim:
                out[:, d] = (u01(r[k]) * np.float32(w[d])).astype(np.float32) + np.float32(lo[d])
    return out
