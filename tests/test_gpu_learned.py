"""Learned control variate: the network's forward/backward kernels against the FP64 reference
(oracle/mlp_ref.py, which rounds to BF16 at the same points), and what training buys.

Tolerances: outputs within 2e-3 relative (L2) of the reference and gradients within 2e-2 relative
(L2) with cosine similarity > 0.999 -- the device accumulates BF16 products in FP32 in a different
order, and its sinpi/cospi features can round to a neighbouring BF16 value."""
import numpy as np
import pytest

from oracle import mlp_ref
from viltrum_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim", [2, 3, 5])
def test_forward_backward_against_fp64_reference(ctx, dim):
    rng = np.random.default_rng(dim)
    theta = mlp_ref.init(dim, seed=10 + dim)
    # non-zero biases exercise every parameter's gradient
    theta = (theta + rng.normal(0, 0.05, theta.size).astype(np.float32)).astype(np.float32)
    n = 3000
    u = rng.random((n, dim)).astype(np.float32)
    y = rng.normal(0, 1, n).astype(np.float32)
    out, grad = ctx.mlp_eval(dim, theta, u, y, grad=True)
    ref_out, ref_grad = mlp_ref.forward_backward(theta, u.astype(np.float64), y.astype(np.float64))
    rel_out = np.linalg.norm(out - ref_out) / np.linalg.norm(ref_out)
    assert rel_out < 2e-3, rel_out
    rel_g = np.linalg.norm(grad - ref_grad) / np.linalg.norm(ref_grad)
    cos = float(np.dot(grad, ref_grad) / (np.linalg.norm(grad) * np.linalg.norm(ref_grad)))
    assert rel_g < 2e-2 and cos > 0.999, (rel_g, cos)
    # every layer's block of the gradient agrees, not just the total
    f = mlp_ref.fin(dim)
    blocks = [(0, f * 64), (f * 64 + 64, f * 64 + 64 + 4096), (len(grad) - 65, len(grad))]
    for a, b in blocks:
        gb, rb = grad[a:b], ref_grad[a:b]
        assert np.linalg.norm(gb - rb) <= 3e-2 * np.linalg.norm(rb) + 1e-7


def _learned(ctx, kind, params, rmin, rmax, res, spp, seed, steps, fallback=0, q=3, lr=2e-3, batch=32768, cells=1):
    p = ctx.problem(kind, params, rmin, rmax, res)
    nb = int(np.prod(res))
    out = np.empty(nb, np.float32)
    integ = np.empty(nb, np.float32)
    opts = _lib.LearnedOpts(spp, seed, steps, batch, lr, q, fallback, cells)
    st, rep = ctx.learned_control_variates(p, opts, out, integ)
    return out, integ, st, rep


def test_training_gain_over_plain_monte_carlo(ctx):
    """On the smooth sin(8x)e^-y + x^2 + y^2 over coarse 8x8 bins (where the integrand varies a lot
    inside a bin, so plain per-bin Monte Carlo is noisy) the trained network removes most of the
    variance: the learned estimator's bin RMSE is several times lower than plain Monte Carlo's with
    the same residual samples, and than the untrained network's.  (On fine bins the integrand is
    nearly constant inside a bin and the gain shrinks: 1.6x at 64x64 after 1600 steps.)  The network's
    integral over a bin uses 4 cells x 4 Gauss-Legendre nodes per dimension: its frequency features
    reach 32 pi, two periods per 1/8-wide bin."""
    res, spp = [8, 8], 32
    exact = scenes.exact_bins(scenes.WAVE2, None, [0, 0], [1, 1], res)[:, 0]
    trained, integ, st, rep = _learned(ctx, scenes.WAVE2, None, [0, 0], [1, 1], res, spp, 5, steps=1000, lr=3e-3,
                                       q=4, cells=4)
    untrained, _, _, _ = _learned(ctx, scenes.WAVE2, None, [0, 0], [1, 1], res, spp, 5, steps=0, q=4, cells=4)
    p = ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], res)
    mc = np.empty(8 * 8, np.float32)
    ctx.per_bin_monte_carlo(p, spp, 5, mc)
    r_tr = scenes.bin_rmse(trained, exact[:, None])
    r_un = scenes.bin_rmse(untrained, exact[:, None])
    r_mc = scenes.bin_rmse(mc, exact[:, None])
    assert r_tr < 0.25 * r_mc, (r_tr, r_mc)
    assert r_tr < 0.25 * r_un, (r_tr, r_un)
    assert np.isfinite(trained).all() and st.flags == 0
    assert rep.train_ms > 0 and rep.integral_ms > 0 and rep.residual_ms > 0


def test_learned_estimator_is_unbiased(ctx):
    """Mean over seeds of the bin errors is within a few standard errors of zero (the only bias is
    the quadrature error of the network's integral, far below the residual noise)."""
    res, spp = [32, 32], 16
    exact = scenes.exact_bins(scenes.WAVE2, None, [0, 0], [1, 1], res)[:, 0]
    errs = []
    for seed in range(6):
        out, _, _, _ = _learned(ctx, scenes.WAVE2, None, [0, 0], [1, 1], res, spp, 100 + seed, steps=100)
        errs.append(out - exact)
    errs = np.array(errs)
    mean_err = errs.mean()
    se = errs.std() / np.sqrt(errs.size)
    assert abs(mean_err) < 4 * se + 1e-6, (mean_err, se)


def test_occluded_scene_runs_with_fallback(ctx):
    """5-D occluded scene at a small resolution: finite, fallback bins counted, and not worse than
    plain Monte Carlo at the same samples (the per-bin fallback guards against a poor network)."""
    params = scenes.occluded_scene5(7)
    res, spp = [32, 32], 32
    out, integ, st, rep = _learned(ctx, scenes.OCCLUDED_SCENE5, params, [0] * 5, [1] * 5, res, spp, 3, steps=200,
                                   fallback=1, q=2)
    assert np.isfinite(out).all() and np.isfinite(integ).all()
    assert rep.fallback_bins <= 32 * 32
