"""Synthetic integrands of the per-bin integration workloads and their FP64 bin integrals.

Every scene parameter is drawn from one counter-based generator (SplitMix64 -> uniform double in
[0,1), Steele, Lea & Flood, OOPSLA 2014) so that identical parameters reach the CPU and the GPU.
The returned parameter arrays are the flat float32 layouts that vcu_integrands.h documents.

Bin values follow viltrum's normalisation: bin value = (prod of the bin resolution) x integral of
f over the bin (src/integrator-per-bin.h:26, src/monte-carlo/monte-carlo.h:45).
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf

# integrand tags (vcu_integrands.h)
POLY2, SIN1, SPHERE3, WAVE2, SCENE2, MOVING_SCENE3, HALFSPACE, OCCLUDED_SCENE5, WALK2 = 1, 2, 3, 4, 5, 6, 7, 8, 9
DIMS = {POLY2: 2, SIN1: 1, SPHERE3: 3, WAVE2: 2, SCENE2: 2, MOVING_SCENE3: 3, OCCLUDED_SCENE5: 5}
CHANNELS = {MOVING_SCENE3: 3}

_M64 = (1 << 64) - 1


class SplitMix64:
    """SplitMix64 stream; uniform() returns doubles in [0, 1) from the top 53 bits."""

    def __init__(self, seed: int):
        self.state = seed & _M64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & _M64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))


def scene2(seed: int = 7, n_gauss: int = 64, n_disk: int = 32) -> np.ndarray:
    """Gaussian bumps (c ~ U[0,1]^2, sigma ~ U(0.005,0.05), A ~ U(0,1)) plus hard-edged disks
    (c ~ U[0,1]^2, r ~ U(0.01,0.1), value ~ U(0,1))."""
    g = SplitMix64(seed)
    p = [float(n_gauss), float(n_disk)]
    for _ in range(n_gauss):
        p += [g.uniform(), g.uniform(), g.uniform(0.005, 0.05), g.uniform()]
    for _ in range(n_disk):
        p += [g.uniform(), g.uniform(), g.uniform(0.01, 0.1), g.uniform()]
    return np.array(p, dtype=np.float32)


def moving_scene3(seed: int = 7, n_gauss: int = 64, n_disk: int = 32) -> np.ndarray:
    """scene2's bumps (static, grey) and disks whose centres move by velocities U(-0.1,0.1)^2
    over t in [0,1]; each disk carries value x RGB with RGB ~ U(0,1)^3."""
    g = SplitMix64(seed)
    p = [float(n_gauss), float(n_disk)]
    for _ in range(n_gauss):
        p += [g.uniform(), g.uniform(), g.uniform(0.005, 0.05), g.uniform()]
    for _ in range(n_disk):
        cx, cy, r, v = g.uniform(), g.uniform(), g.uniform(0.01, 0.1), g.uniform()
        vx, vy = g.uniform(-0.1, 0.1), g.uniform(-0.1, 0.1)
        rgb = [v * g.uniform() for _ in range(3)]
        p += [cx, cy, vx, vy, r] + rgb
    return np.array(p, dtype=np.float32)


def halfspace(seed: int, dim: int) -> np.ndarray:
    """prod_d exp(-a_d x_d) cos(b_d x_d) [n.x < c]: a ~ U(0,4), b ~ U(0,20), n a random unit
    vector, c ~ U(0, sqrt(dim))."""
    g = SplitMix64(seed)
    a = [g.uniform(0.0, 4.0) for _ in range(6)]
    b = [g.uniform(0.0, 20.0) for _ in range(6)]
    n = np.array([g.uniform(-1.0, 1.0) for _ in range(6)])
    n[dim:] = 0.0
    n = n / np.linalg.norm(n[:dim])
    c = g.uniform(0.0, float(np.sqrt(dim)))
    a = [a[i] if i < dim else 0.0 for i in range(6)]
    b = [b[i] if i < dim else 0.0 for i in range(6)]
    return np.array([float(dim)] + a + b + list(n) + [c], dtype=np.float32)


def batch_items(n: int, seed: int = 11, budget_lo: int = 256, budget_hi: int = 65536, dims=(2, 6),
                methods=(0, 1)) -> list[dict]:
    """The batched-integrals workload: n independent integrals over [0,1]^dim, dim uniform in
    dims[0]..dims[1], integrand the half-space family (seeded per item), method drawn uniformly
    from `methods` (0 Monte Carlo, 1 adaptive nested), budget log-uniform in [budget_lo, budget_hi]
    (samples or regions), Monte Carlo seed per item."""
    g = SplitMix64(seed)
    items = []
    lo, hi = np.log(budget_lo), np.log(budget_hi)
    for i in range(n):
        dim = dims[0] + min(int(g.uniform() * (dims[1] - dims[0] + 1)), dims[1] - dims[0])
        method = methods[min(int(g.uniform() * len(methods)), len(methods) - 1)]
        budget = int(round(float(np.exp(lo + (hi - lo) * g.uniform()))))
        budget = max(budget_lo, min(budget_hi, budget))
        item_seed = g.next_u64() & 0xFFFFFFFF
        items.append(dict(dim=dim, method=method, budget=budget, seed=item_seed,
                          params=halfspace(seed * 1000003 + i, dim), rmin=[0.0] * dim, rmax=[1.0] * dim))
    return items


def walk2(seed: int = 7, n_gauss: int = 16, n_disk: int = 8, albedo: float = 0.6, keep: float = 0.7,
          step: float = 0.15, max_bounces: int = 32, key: int = 11) -> np.ndarray:
    """The random walk over scene2(seed): an integrand of unbounded dimension (vcu_integrands.h
    Walk2): [albedo, keep, step, max_bounces, key] then the scene's parameters."""
    return np.concatenate([np.array([albedo, keep, step, max_bounces, key], np.float32),
                           scene2(seed, n_gauss, n_disk)]).astype(np.float32)


def occluded_scene5(seed: int = 7, n_gauss: int = 64, n_disk: int = 32, n_box: int = 128) -> np.ndarray:
    """scene2 followed by n_box occluder boxes: centre ~ U[0,1]^3, half-size ~ U(0.01,0.08)^3."""
    s = list(scene2(seed, n_gauss, n_disk).astype(np.float64))
    g = SplitMix64(seed ^ 0x5DEECE66D)
    s.append(float(n_box))
    for _ in range(n_box):
        s += [g.uniform(), g.uniform(), g.uniform()] + [g.uniform(0.01, 0.08) for _ in range(3)]
    return np.array(s, dtype=np.float32)


# ---------------------------------------------------------------------------- FP64 bin integrals
def _edges(rmin, rmax, res):
    return [np.linspace(float(rmin[d]), float(rmax[d]), int(res[d]) + 1) for d in range(len(res))]


def _bins_grid(rmin, rmax, res):
    """x0, x1, y0, y1 arrays of shape (nbins,), bins dim-0-fastest."""
    ex, ey = _edges(rmin, rmax, res)
    x0, y0 = np.meshgrid(ex[:-1], ey[:-1], indexing="xy")
    x1, y1 = np.meshgrid(ex[1:], ey[1:], indexing="xy")
    return x0.ravel(), x1.ravel(), y0.ravel(), y1.ravel()


def _gauss_1d(a, b, c, s):
    k = 1.0 / (s * np.sqrt(2.0))
    return s * np.sqrt(np.pi / 2.0) * (erf((b - c) * k) - erf((a - c) * k))


def _corner(a, b, r):
    """Area of the disk x^2+y^2<=r^2 inside the rectangle spanned by (0,0) and (a,b), signed."""
    sa, sb = np.sign(a), np.sign(b)
    a = np.minimum(np.abs(a), r)
    b = np.minimum(np.abs(b), r)
    inside = a * a + b * b <= r * r
    xs = np.sqrt(np.maximum(r * r - b * b, 0.0))
    xs = np.minimum(xs, a)

    def prim(x):
        return 0.5 * (x * np.sqrt(np.maximum(r * r - x * x, 0.0)) + r * r * np.arcsin(np.clip(x / r, -1.0, 1.0)))

    outside = b * xs + prim(a) - prim(xs)
    return sa * sb * np.where(inside, a * b, outside)


def disk_rect_area(cx, cy, r, x0, x1, y0, y1):
    """Exact area of disk((cx,cy), r) intersected with [x0,x1]x[y0,y1] (broadcasting)."""
    X0, X1, Y0, Y1 = x0 - cx, x1 - cx, y0 - cy, y1 - cy
    return _corner(X1, Y1, r) - _corner(X0, Y1, r) - _corner(X1, Y0, r) + _corner(X0, Y0, r)


def exact_bins(kind: int, params, rmin, rmax, res, t_nodes: int = 48) -> np.ndarray:
    """FP64 bin values (prod(res) x integral over the bin), shape (nbins, channels)."""
    res = [int(r) for r in res]
    nb = int(np.prod(res))
    factor = float(np.prod(res))
    if kind in (WAVE2, POLY2):
        if len(res) == 1:
            ex = _edges(rmin, rmax, res)[0]
            x0, x1 = ex[:-1], ex[1:]
            y0 = np.full_like(x0, float(rmin[1]))
            y1 = np.full_like(x0, float(rmax[1]))
        else:
            x0, x1, y0, y1 = _bins_grid(rmin, rmax, res)
        v = (x1 ** 3 - x0 ** 3) / 3.0 * (y1 - y0) + (y1 ** 3 - y0 ** 3) / 3.0 * (x1 - x0)
        if kind == WAVE2:
            v = v + (np.cos(8 * x0) - np.cos(8 * x1)) / 8.0 * (np.exp(-y0) - np.exp(-y1))
        return (factor * v).reshape(nb, 1)
    if kind == SIN1:
        ex = _edges(rmin, rmax, res)[0]
        return (factor * (np.cos(ex[:-1]) - np.cos(ex[1:]))).reshape(nb, 1)
    if kind in (SCENE2, MOVING_SCENE3):
        p = np.asarray(params, dtype=np.float64)
        ng, nd = int(p[0]), int(p[1])
        g = p[2:2 + 4 * ng].reshape(ng, 4)
        if len(res) == 1:
            ex = _edges(rmin, rmax, res)[0]
            x0, x1 = ex[:-1], ex[1:]
            y0 = np.full_like(x0, float(rmin[1]))
            y1 = np.full_like(x0, float(rmax[1]))
        else:
            x0, x1, y0, y1 = _bins_grid(rmin, rmax, res)
        grey = np.zeros(nb)
        for cx, cy, s, a in g:
            grey += a * _gauss_1d(x0, x1, cx, s) * _gauss_1d(y0, y1, cy, s)
        if kind == SCENE2:
            d = p[2 + 4 * ng:2 + 4 * ng + 4 * nd].reshape(nd, 4)
            v = grey.copy()
            for cx, cy, r, val in d:
                v += val * disk_rect_area(cx, cy, r, x0, x1, y0, y1)
            return (factor * v).reshape(nb, 1)
        # moving disks: integrate the exact area over t with composite Gauss-Legendre
        d = p[2 + 4 * ng:2 + 4 * ng + 8 * nd].reshape(nd, 8)
        t0, t1 = float(rmin[2]), float(rmax[2])
        gx, gw = np.polynomial.legendre.leggauss(8)
        panels = max(1, t_nodes // 8)
        edges = np.linspace(t0, t1, panels + 1)
        out = np.repeat(grey[:, None] * (t1 - t0), 3, axis=1)
        for cx, cy, vx, vy, r, cr, cg, cb in d:
            acc = np.zeros(nb)
            for pa, pb in zip(edges[:-1], edges[1:]):
                for xi, wi in zip(gx, gw):
                    t = 0.5 * (pa + pb) + 0.5 * (pb - pa) * xi
                    acc += 0.5 * (pb - pa) * wi * disk_rect_area(cx + t * vx, cy + t * vy, r, x0, x1, y0, y1)
            out += acc[:, None] * np.array([cr, cg, cb])[None, :]
        return factor * out
    raise ValueError(f"no FP64 bin integrals for integrand kind {kind}")


def bin_rmse(est, truth) -> float:
    est = np.asarray(est, dtype=np.float64).reshape(np.asarray(truth).shape)
    return float(np.sqrt(np.mean((est - truth) ** 2)))
