"""Known answers of the reference's own checks of single pieces, held by the CPU oracle.

* main/compilation-tests/covariance.cc:38-50 -- the control-variate weight accumulator's online
  variance and covariance (shifted by the first sample) equal the two-pass ones.
* main/compilation-tests/region-sample.cc:25-52 -- a Simpson region's pdf integrates to one, and its
  sampler draws a histogram that follows the pdf.
* main/compilation-tests/inverse.cc:60-88 -- the inverse cdf of the Simpson parabola over a narrow
  sub-range returns one point inside it for every uniform draw.

Where oracle/_ref (the unmodified reference) is built, the same probes are also compared with it
bit for bit on random inputs; the committed fixture pieces_cv_moments_simpson_pdf.npz pins them
everywhere else (tests/test_oracle_golden.py)."""
import numpy as np
import pytest

from oracle import oracle as orc


def _cdf(nodes, t):
    """FP64 cdf of the parabola through (0, n0), (0.5, n1), (1, n2), from 0 to t."""
    n0, n1, n2 = (float(v) for v in nodes)
    c0, c1, c2 = n0, -3 * n0 + 4 * n1 - n2, 2 * n0 - 4 * n1 + 2 * n2
    t = np.asarray(t, np.float64)
    return ((c2 * t / 3 + c1 / 2) * t + c0) * t


@pytest.mark.parametrize("n,noise", [(20, 0.1), (2000, 0.5)])
def test_online_covariance_matches_two_pass(port, n, noise):
    rng = np.random.default_rng(n)
    g = np.sin(rng.uniform(0, 2 * np.pi, n)).astype(np.float32)
    f = (g + rng.uniform(-noise, noise, n)).astype(np.float32)
    var, cov, alpha, integral = port.cv_optimize_moments(f, g, approximation=0.5)
    # the accumulator works on the norms (absolute values) and divides by n - 1
    a, b = np.abs(f.astype(np.float64)), np.abs(g.astype(np.float64))
    var2 = ((b - b.mean()) ** 2).sum() / (n - 1)
    cov2 = ((a - a.mean()) * (b - b.mean())).sum() / (n - 1)
    assert var == pytest.approx(var2, rel=1e-5)
    assert cov == pytest.approx(cov2, rel=1e-5, abs=1e-9)
    assert alpha == pytest.approx(min(var2, max(0.0, cov2)) / var2, rel=1e-5)
    assert integral == pytest.approx((f.sum(dtype=np.float64) - alpha * g.sum(dtype=np.float64)) / n + alpha * 0.5,
                                     rel=1e-5)


def test_accumulator_edge_cases(port):
    g = np.linspace(0.1, 0.9, 50, dtype=np.float32)
    # no variance in the approximation: alpha 1
    assert port.cv_optimize_moments(g, np.full(50, 0.3, np.float32))[2] == 1.0
    # norms anti-correlated: alpha clamps to 0, the estimate is the plain mean
    _, cov, alpha, integral = port.cv_optimize_moments((1.5 - g).astype(np.float32), g, 2.0)
    assert cov < 0 and alpha == 0.0
    assert integral == pytest.approx(float((1.5 - g).astype(np.float32).mean(dtype=np.float64)), rel=1e-6)
    # one sample: the estimate is the approximation
    assert port.cv_optimize_moments(g[:1], g[1:2], 0.7)[3] == pytest.approx(0.7, rel=1e-7)


def test_simpson_pdf_follows_histogram(port):
    nodes = np.array([1.0, 0.2, 1.0], np.float32)  # region-sample.cc's default parabola
    for lo, hi in ((0.0, 1.0), (0.2, 0.9)):
        bins = 6
        edges = np.linspace(lo, hi, bins + 1)
        centres = (edges[:-1] + edges[1:]) / 2
        probs = port.simpson_pdf_1d(nodes, centres, lo, hi)
        # the pdf at a point is the parabola over its integral on [lo, hi]
        n0, n1, n2 = (float(v) for v in nodes)
        c1, c2 = -3 * n0 + 4 * n1 - n2, 2 * n0 - 4 * n1 + 2 * n2
        exact = np.diff(_cdf(nodes, [lo, hi]))[0]
        assert np.allclose(probs, (n0 + c1 * centres + c2 * centres ** 2) / exact, rtol=1e-5)
        # so its midpoint sum plus the midpoint rule's error on a parabola (h^2/24 f'' per unit length) is one
        h = (hi - lo) / bins
        assert (probs * h).sum() + h * h / 24 * 2 * c2 * (hi - lo) / exact == pytest.approx(1.0, abs=1e-5)
        # samples fall where the pdf puts its mass: per-bin counts within 5 sigma of the cdf's share
        samples = 50_000
        s = np.random.default_rng(3).uniform(0, 1, samples).astype(np.float32)
        x = port.simpson_sample_1d(nodes, s, lo, hi)
        assert x.min() >= np.float32(lo) and x.max() <= np.float32(hi)
        hist = np.histogram(x, bins=edges)[0]
        share = np.diff(_cdf(nodes, edges)) / exact
        sigma = np.sqrt(samples * share * (1 - share))
        assert np.all(np.abs(hist - samples * share) <= 5 * sigma + 1)


def test_inverse_cdf_in_narrow_range(port):
    nodes = np.array([0.43, 0.9, 0.42], np.float32)  # inverse.cc's parabola
    a, b = 0.0, 0.125
    s = (np.arange(10) * np.float32(0.1)).astype(np.float32)
    x = port.simpson_sample_1d(nodes, s, a, b)
    assert np.all((x >= a) & (x <= b))
    assert np.all(np.diff(x) > 0)
    target = _cdf(nodes, a) + s.astype(np.float64) * (_cdf(nodes, b) - _cdf(nodes, a))
    assert np.allclose(_cdf(nodes, x), target, atol=1e-6)


def test_pieces_match_reference_on_random_inputs(port):
    ref = orc.reference()
    if ref is None:
        pytest.skip("oracle/_ref is not built (needs the reference sources)")
    rng = np.random.default_rng(99)
    for _ in range(20):
        n = int(rng.integers(2, 300))
        f = rng.normal(0, 1, n).astype(np.float32)
        g = (f * rng.uniform(-1, 1) + rng.normal(0, 0.3, n)).astype(np.float32)
        r, p = ref.cv_optimize_moments(f, g, 0.25), port.cv_optimize_moments(f, g, 0.25)
        assert np.array_equal(np.array(r).view(np.uint64), np.array(p).view(np.uint64))
    for _ in range(40):
        nodes = rng.uniform(-1, 2, 3).astype(np.float32)
        t0 = float(np.float32(rng.uniform(0, 0.5)))
        t1 = float(np.float32(t0 + rng.uniform(0.01, 0.5)))
        t = np.linspace(t0, t1, 7).astype(np.float32)
        s = rng.uniform(0, 1, 7).astype(np.float32)
        for fn in ("simpson_pdf_1d", "simpson_sample_1d"):
            u = t if fn == "simpson_pdf_1d" else s
            rv, pv = getattr(ref, fn)(nodes, u, t0, t1), getattr(port, fn)(nodes, u, t0, t1)
            assert np.array_equal(rv.view(np.uint32), pv.view(np.uint32)), (fn, nodes, t0, t1)
