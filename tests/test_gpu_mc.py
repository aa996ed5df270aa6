"""Per-bin Monte Carlo: replay parity against the reference's own sample points, exact
reproduction of the device's Philox points, and statistics of the Philox estimator against the
FP64 closed form.

Replay tolerance: the reference accumulates `sol += f*factor` in float (src/monte-carlo/monte-carlo.h:59),
so its bin value is within n*u*sum|terms| (u = 2^-24) of the exact sum of the same terms; the GPU
sums in compensated FP32 and must be within 1e-6 relative of the FP64 sum of the same points and
within the reference's own float-accumulation bound of the reference value."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
import philox_np
from viltrum_gb300 import scenes

pytestmark = pytest.mark.gpu
U = 2.0 ** -24


def _bins_geometry(rmin, rmax, res, dim):
    """per-bin lower corner and widths (float32, as the reference computes them)"""
    rmin = np.asarray(rmin, np.float32)
    rmax = np.asarray(rmax, np.float32)
    nb = int(np.prod(res))
    lo = np.tile(rmin, (nb, 1))
    w = np.tile(rmax - rmin, (nb, 1))
    lin = np.arange(nb)
    for d, r in enumerate(res):
        pos = (lin % r).astype(np.float32)
        lin = lin // r
        dr = np.float32(rmax[d] - rmin[d]) / np.float32(r)
        a = rmin[d] + pos * dr
        b = rmin[d] + (pos + np.float32(1)) * dr
        lo[:, d] = a
        w[:, d] = (b - a).astype(np.float32)
    return lo.astype(np.float32), w.astype(np.float32)


@pytest.mark.parametrize("name", golden_names("mc_"))
def test_replay_matches_reference(ctx, port, name):
    g = load_golden(name)
    if "out_points" not in g:
        pytest.skip("fixture without recorded points")
    kind, res, spp = int(g["kind"]), [int(r) for r in g["res"]], int(g["spp"])
    pts = np.ascontiguousarray(g["out_points"], np.float32)
    dim = pts.shape[2]
    p = ctx.problem(kind, g.get("params"), g["rmin"], g["rmax"], res)
    nb = int(np.prod(res))
    ch = 3 if kind == scenes.MOVING_SCENE3 else 1
    fvals = port.eval(kind, g.get("params"), pts.reshape(-1, dim)).reshape(nb, spp, ch).astype(np.float64)
    if int(g["flavour"]) == 0:
        # integrator_per_bin_parallel(monte_carlo): prod(res) * volume(bin) / spp * sum f, assigned
        out = np.empty(nb * ch, np.float32)
        ctx.per_bin_monte_carlo_replay(p, spp, pts, out)
        lo, w = _bins_geometry(g["rmin"], g["rmax"], res, dim)
        vol = np.prod(w.astype(np.float32), axis=1, dtype=np.float32).astype(np.float64)
        factor = float(np.prod(res)) * vol / spp
    else:
        # monte_carlo_per_bin_parallel (monte-carlo-per-bin-parallel.h:45,69): bins (zero here, as
        # in the fixture) += volume(range) / spp * f per sample
        out = np.zeros(nb * ch, np.float32)
        ctx.per_bin_monte_carlo_accumulate(p, spp, 0, out, points=pts)
        width = np.asarray(g["rmax"], np.float32) - np.asarray(g["rmin"], np.float32)
        factor = np.full(nb, float(np.prod(width, dtype=np.float32)) / spp)
    out = out.reshape(nb, ch).astype(np.float64)
    exact = fvals.sum(axis=1) * factor[:, None]
    assert np.all(np.abs(out - exact) <= 1e-6 * np.abs(exact) + 1e-12)
    ref = g["out_bins"].astype(np.float64)
    bound = spp * U * np.abs(fvals).sum(axis=1) * factor[:, None] + 2 * U * np.abs(ref)
    assert np.all(np.abs(out - ref) <= bound + 1e-12)


def test_philox_points_reproduced_exactly(ctx, port):
    """The device estimate equals the FP64 sum over the points a CPU Philox predicts."""
    kind, res, spp, seed = scenes.WAVE2, [37], 300, 0x1234_5678_9ABC
    p = ctx.problem(kind, None, [0, 0], [1, 1], res)
    out = np.empty(37, np.float32)
    ctx.per_bin_monte_carlo(p, spp, seed, out)
    lo, w = _bins_geometry([0, 0], [1, 1], res, 2)
    for b in (0, 5, 36):
        pts = philox_np.points(b, spp, 2, seed, lo[b], w[b])
        f = port.eval(kind, None, pts)[:, 0].astype(np.float64)
        est = 37 * float(np.prod(w[b], dtype=np.float32)) / spp * f.sum()
        assert abs(out[b] - est) <= 1e-6 * abs(est)


def test_philox_deterministic_and_seeded(ctx):
    p = ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], [256])
    a, b, c = (np.empty(256, np.float32) for _ in range(3))
    ctx.per_bin_monte_carlo(p, 64, 9, a)
    ctx.per_bin_monte_carlo(p, 64, 9, b)
    ctx.per_bin_monte_carlo(p, 64, 10, c)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert not np.array_equal(a, c)


def test_philox_statistics_against_fp64(ctx, port):
    """1024 bins x 1024 samples of sin(8x)e^-y + x^2 + y^2: per-bin errors against the closed form
    are consistent with the per-bin sampling sigma (mean of z ~ 0, few 3-sigma exceedances), and the
    mean squared error matches the reference estimator's at equal samples (ratio in [0.8, 1.25])."""
    res, spp = [1024], 1024
    exact = scenes.exact_bins(scenes.WAVE2, None, [0, 0], [1, 1], res)[:, 0]
    # per-bin variance of f from a dense stratified evaluation
    lo, w = _bins_geometry([0, 0], [1, 1], res, 2)
    rng = np.random.default_rng(0)
    u = rng.random((1024, 512, 2)).astype(np.float32)
    x = (lo[:, None, :] + u * w[:, None, :]).astype(np.float32)
    fv = port.eval(scenes.WAVE2, None, x.reshape(-1, 2))[:, 0].reshape(1024, 512).astype(np.float64)
    sigma = np.sqrt(fv.var(axis=1, ddof=1) / spp)
    p = ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], res)
    gpu_sq, ref_sq = [], []
    for seed in (1, 2, 3):
        out = np.empty(1024, np.float32)
        ctx.per_bin_monte_carlo(p, spp, seed, out)
        z = (out - exact) / sigma
        assert abs(z.mean()) < 0.2
        assert (np.abs(z) > 3).sum() <= 12
        gpu_sq.append(np.mean((out - exact) ** 2))
        ref, _ = port.per_bin_monte_carlo(scenes.WAVE2, None, [0, 0], [1, 1], res, spp, seed)
        ref_sq.append(np.mean((ref[:, 0] - exact) ** 2))
    ratio = np.mean(gpu_sq) / np.mean(ref_sq)
    assert 0.8 <= ratio <= 1.25


def test_accumulating_flavour_adds_to_current_values(ctx, port):
    """monte_carlo_per_bin_parallel adds volume(range)/spp * sum f to whatever the bins hold: the
    oracle's own points replayed onto a non-zero start equal start + the oracle's zero-start bins
    (within the reference's float-accumulation bound)."""
    res, spp = [6, 5], 32
    start = np.linspace(-2.0, 3.0, 30, dtype=np.float32)
    ref0, pts = port.per_bin_monte_carlo(scenes.WAVE2, None, [0, -1], [2, 1], res, spp, 4, flavour=1, record=True)
    ref, _ = port.per_bin_monte_carlo(scenes.WAVE2, None, [0, -1], [2, 1], res, spp, 4, flavour=1,
                                      initial=start)
    p = ctx.problem(scenes.WAVE2, None, [0, -1], [2, 1], res)
    out = start.copy()
    ctx.per_bin_monte_carlo_accumulate(p, spp, 0, out, points=np.ascontiguousarray(pts))
    fv = port.eval(scenes.WAVE2, None, pts.reshape(-1, 2))[:, 0].reshape(30, spp).astype(np.float64)
    exact = start.astype(np.float64) + fv.sum(axis=1) * 4.0 / spp
    assert np.all(np.abs(out - exact) <= 2 * U * np.abs(exact) + 1e-12)
    bound = (spp + 1) * U * (np.abs(fv).sum(axis=1) * 4.0 / spp + np.abs(start))
    assert np.all(np.abs(out - ref[:, 0]) <= bound)


def test_accumulating_flavour_and_rgb(ctx, port):
    """monte_carlo_per_bin_parallel adds into the caller's bins; RGB integrands fill 3 channels."""
    import viltrum_gb300 as v
    bins = np.ones((8, 8, 3), np.float32)
    params = scenes.moving_scene3(7, n_gauss=8, n_disk=8)
    v.integrate(v.monte_carlo_per_bin_parallel(4096, 3), bins, v.Integrand.moving_scene3(params),
                v.range_primary(3), ctx=ctx)
    exact = scenes.exact_bins(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], [8, 8], t_nodes=96)
    est = bins.reshape(8, 8, 3).transpose(1, 0, 2).reshape(64, 3) - 1.0
    assert np.sqrt(np.mean((est - exact) ** 2)) < 0.05
