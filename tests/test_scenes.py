"""Synthetic workloads: generator determinism, portable math accuracy, FP64 bin integrals."""
import numpy as np
from scipy import integrate as si

from viltrum_gb300 import scenes


def test_splitmix64_known_values():
    # first outputs of SplitMix64 seeded with 0 (Steele, Lea & Flood's reference sequence)
    g = scenes.SplitMix64(0)
    assert g.next_u64() == 0xE220A8397B1DCDAF
    assert g.next_u64() == 0x6E789E6AA1B965F4
    assert g.next_u64() == 0x06C45D188009454F


def test_scene_layout():
    p = scenes.scene2(7)
    assert p.dtype == np.float32 and p.size == 2 + 4 * 64 + 4 * 32
    assert np.array_equal(p, scenes.scene2(7)) and not np.array_equal(p, scenes.scene2(8))
    s = p[2:2 + 256].reshape(64, 4)
    assert (s[:, 2] >= 0.005).all() and (s[:, 2] <= 0.05).all()


def test_portable_math_accuracy(port):
    """vexp/vsin/vcos (vcu_integrands.h) against numpy's double results, through the oracle."""
    x = np.linspace(-20, 20, 20001, dtype=np.float32)
    # SIN1 integrand evaluates vsin
    s = port.eval(scenes.SIN1, None, x[:, None])[:, 0]
    assert np.max(np.abs(s - np.sin(x.astype(np.float64)))) < 4e-7
    # WAVE2 at x=0 is exp(-y) * sin(0) + y^2 -> use x small to isolate: f(x,0) = sin(8x) + x^2
    xs = np.linspace(0, 1, 4001, dtype=np.float32)
    w = port.eval(scenes.WAVE2, None, np.stack([xs, np.zeros_like(xs)], 1))[:, 0]
    ref = np.sin(8 * xs.astype(np.float64)) + xs.astype(np.float64) ** 2
    assert np.max(np.abs(w - ref)) < 1e-6
    ys = np.linspace(0, 1, 4001, dtype=np.float32)
    w = port.eval(scenes.WAVE2, None, np.stack([np.full_like(ys, 0.19634954), ys], 1))[:, 0]  # sin(8x)=1
    ref = np.sin(8 * np.float64(np.float32(0.19634954))) * np.exp(-ys.astype(np.float64)) + \
        np.float64(np.float32(0.19634954)) ** 2 + ys.astype(np.float64) ** 2
    assert np.max(np.abs(w - ref) / np.abs(ref)) < 3e-7


def test_disk_rect_area_matches_quadrature():
    rng = np.random.default_rng(0)
    for _ in range(20):
        cx, cy, r = rng.uniform(0, 1), rng.uniform(0, 1), rng.uniform(0.01, 0.3)
        x0, y0 = rng.uniform(0, 1, 2)
        x1, y1 = x0 + rng.uniform(0.01, 0.5), y0 + rng.uniform(0.01, 0.5)

        def chord(x):
            h = np.sqrt(max(r * r - (x - cx) ** 2, 0.0))
            return max(0.0, min(y1, cy + h) - max(y0, cy - h))

        q, _ = si.quad(chord, x0, x1, points=[cx - r, cx + r], limit=200, epsabs=1e-13)
        assert abs(scenes.disk_rect_area(cx, cy, r, x0, x1, y0, y1) - q) < 1e-10


def test_exact_bins_scene_against_quadrature(port):
    """FP64 closed-form bin values of the scene against adaptive quadrature of the integrand."""
    p = scenes.scene2(7)
    res = [8, 8]
    ex = scenes.exact_bins(scenes.SCENE2, p, [0, 0], [1, 1], res)
    assert ex.shape == (64, 1)
    # total over the domain: sum(bins)/prod(res) = integral over [0,1]^2, check against bin sums of a
    # finer exact grid (consistency) and a dense midpoint evaluation of the oracle integrand
    fine = scenes.exact_bins(scenes.SCENE2, p, [0, 0], [1, 1], [64, 64])
    assert abs(ex.sum() / 64 - fine.sum() / 4096) < 1e-12
    n = 1024
    g = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(g, g, indexing="xy")
    vals = port.eval(scenes.SCENE2, p, np.stack([X.ravel(), Y.ravel()], 1).astype(np.float32))[:, 0]
    assert abs(vals.mean() - fine.sum() / 4096) < 2e-4


def test_exact_bins_wave2_closed_form():
    ex = scenes.exact_bins(scenes.WAVE2, None, [0, 0], [1, 1], [4])
    for i in range(4):
        x0, x1 = i / 4, (i + 1) / 4
        q, _ = si.dblquad(lambda y, x: np.sin(8 * x) * np.exp(-y) + x * x + y * y, x0, x1, 0, 1)
        assert abs(ex[i, 0] - 4 * q) < 1e-9
