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


@pytest.mark.parametrize("dim", [2, 3, 5])
def test_tensor_core_forward_against_fp64_reference(ctx, dim):
    """The forward-only path (tcgen05.mma into TMEM, k_mlp_tc.cuh) -- what the learned control variate
    evaluates its grid nodes with -- against the FP64 reference and against the training kernel's
    own forward outputs (mma.sync), on a point count that leaves a partial 128-point tile."""
    rng = np.random.default_rng(100 + dim)
    theta = (mlp_ref.init(dim, seed=20 + dim) + rng.normal(0, 0.05, mlp_ref.n_params(dim))).astype(np.float32)
    n = 3000
    u = rng.random((n, dim)).astype(np.float32)
    out, _ = ctx.mlp_eval(dim, theta, u)
    ref_out, _ = mlp_ref.forward_backward(theta, u.astype(np.float64), np.zeros(n))
    assert np.isfinite(out).all()
    rel = np.linalg.norm(out - ref_out) / np.linalg.norm(ref_out)
    assert rel < 2e-3, rel
    train_out, _ = ctx.mlp_eval(dim, theta, u, np.zeros(n, np.float32), grad=True)
    assert np.linalg.norm(out - train_out) / np.linalg.norm(train_out) < 2e-3


def _learned(ctx, kind, params, rmin, rmax, res, spp, seed, steps, fallback=0, lr=2e-3, batch=32768, cells=0,
             cells_unbinned=2, check_every=0, poly=None, pilot=0):
    p = ctx.problem(kind, params, rmin, rmax, res)
    nb = int(np.prod(res))
    out = np.empty(nb, np.float32)
    integ = np.empty(nb, np.float32)
    pb = pv = None
    if poly is not None:
        pb, pv = (np.ascontiguousarray(a, np.float32) for a in poly)
    opts = _lib.LearnedOpts(spp, seed, steps, batch, lr, check_every, fallback, cells, None, cells_unbinned, pilot,
                            None if pb is None else pb.ctypes.data, None if pv is None else pv.ctypes.data)
    st, rep = ctx.learned_control_variates(p, opts, out, integ)
    return out, integ, st, rep


def _mc_truth(ctx, kind, params, dim, res, spp=1 << 18, reps=4):
    """per-bin truth by plain Monte Carlo, and the mean squared standard error of that truth"""
    p = ctx.problem(kind, params, [0] * dim, [1] * dim, res)
    nb = int(np.prod(res))
    runs = []
    for k in range(reps):
        b = np.empty(nb, np.float32)
        ctx.per_bin_monte_carlo(p, spp, 7000 + k, b)
        runs.append(b.astype(np.float64))
    runs = np.array(runs)
    return runs.mean(axis=0), float(np.mean(runs.var(axis=0, ddof=1) / reps))


def test_training_gain_over_plain_monte_carlo(ctx):
    """On the smooth sin(8x)e^-y + x^2 + y^2 over coarse 8x8 bins (where the integrand varies a lot
    inside a bin, so plain per-bin Monte Carlo is noisy) the trained network's interpolant removes
    most of the variance: the learned estimator's bin RMSE is several times lower than plain Monte
    Carlo's with the same residual samples, and than the untrained network's.  The interpolant uses
    4 Simpson cells per dimension inside each 1/8-wide bin."""
    res, spp = [8, 8], 32
    exact = scenes.exact_bins(scenes.WAVE2, None, [0, 0], [1, 1], res)[:, 0]
    trained, integ, st, rep = _learned(ctx, scenes.WAVE2, None, [0, 0], [1, 1], res, spp, 5, steps=1000, lr=3e-3,
                                       cells=4)
    untrained, _, _, _ = _learned(ctx, scenes.WAVE2, None, [0, 0], [1, 1], res, spp, 5, steps=0, cells=4)
    p = ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], res)
    mc = np.empty(8 * 8, np.float32)
    ctx.per_bin_monte_carlo(p, spp, 5, mc)
    r_tr = scenes.bin_rmse(trained, exact[:, None])
    r_un = scenes.bin_rmse(untrained, exact[:, None])
    r_mc = scenes.bin_rmse(mc, exact[:, None])
    assert r_tr < 0.25 * r_mc, (r_tr, r_mc)
    assert r_tr < 0.25 * r_un, (r_tr, r_un)
    assert np.isfinite(trained).all() and st.flags == 0
    assert rep.nodes_per_bin == 81 and rep.train_steps_run == 1000
    assert rep.train_ms > 0 and rep.integral_ms > 0 and rep.residual_ms > 0


def test_interpolant_integral_is_the_simpson_sum_of_the_network(ctx):
    """network_integral is the composite Simpson mean of the trained network over each bin's grid:
    recomputed on the host from the returned parameters (the network evaluated by vcu_mlp_eval at
    the same nodes), it agrees to FP32 rounding."""
    res = [4, 3]
    nb = 12
    theta = np.empty(mlp_ref.n_params(2), np.float32)
    p = ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], res)
    out = np.empty(nb, np.float32)
    integ = np.empty(nb, np.float32)
    opts = _lib.LearnedOpts(16, 3, 200, 16384, 3e-3, 0, 0, 2, theta.ctypes.data, 1)
    ctx.learned_control_variates(p, opts, out, integ)
    n = 5  # 2 cells -> 5 nodes per dimension
    w = np.array([1, 4, 2, 4, 1], np.float64) / 12.0
    for b in range(nb):
        ix, iy = b % 4, b // 4
        xs = (np.float32(ix) * np.float32(0.25) + (np.float32(0.25)) * np.arange(n, dtype=np.float32) / np.float32(4))
        ys = (np.float32(iy) * np.float32(1 / 3) + np.float32(1 / 3) * np.arange(n, dtype=np.float32) / np.float32(4))
        X, Y = np.meshgrid(xs, ys, indexing="xy")
        u = np.stack([X.ravel(), Y.ravel()], 1).astype(np.float32)
        g = ctx.mlp_eval(2, theta, u)[0].reshape(n, n).astype(np.float64)
        host = float(w @ g @ w)
        assert abs(host - integ[b]) <= 1e-5 * max(1.0, abs(host)), (b, host, integ[b])


@pytest.mark.parametrize("fallback", [0, 1])
def test_learned_estimator_is_unbiased_on_the_occluded_scene(ctx, fallback):
    """The interpolant's integral is exact, so the learned estimator is unbiased even where the
    network fits the integrand poorly (the 5-D occluded scene, whose visibility is discontinuous),
    with weight 1 and with the per-bin weight the pilot fixes before the residual samples: over 8
    seeds the mean error against a Monte Carlo truth is within 4 standard errors of zero."""
    params = scenes.occluded_scene5(7)
    res, spp = [8, 8], 64
    truth, se2 = _mc_truth(ctx, scenes.OCCLUDED_SCENE5, params, 5, res)
    errs = []
    for seed in range(8):
        out, _, st, _ = _learned(ctx, scenes.OCCLUDED_SCENE5, params, [0] * 5, [1] * 5, res, spp, 100 + seed,
                                 steps=60, cells=0, cells_unbinned=2, fallback=fallback)
        assert st.flags == 0
        errs.append(out - truth)
    errs = np.array(errs)
    mean_err = errs.mean()
    se = np.sqrt(errs.var(ddof=1) / errs.size + se2 / errs.shape[1])
    assert abs(mean_err) < 4 * se, (mean_err, se)


def test_learned_beats_plain_monte_carlo_on_the_occluded_scene(ctx):
    """At equal residual samples (32x32 bins of the 5-D occluded scene, 256 samples per bin, the
    interpolant on 4 Simpson cells per primary dimension) the learned estimator's bin RMSE against
    a Monte Carlo truth is below plain Monte Carlo's, and lower still with the per-bin weight the
    pilot estimates (weight 0 in a bin is plain Monte Carlo)."""
    params = scenes.occluded_scene5(7)
    res, spp = [32, 32], 256
    truth, se2 = _mc_truth(ctx, scenes.OCCLUDED_SCENE5, params, 5, res, spp=1 << 16, reps=4)
    p = ctx.problem(scenes.OCCLUDED_SCENE5, params, [0] * 5, [1] * 5, res)

    def rmse(b):
        return float(np.sqrt(max(np.mean((b.astype(np.float64) - truth) ** 2) - se2, 0.0)))

    mc_sq, lr_sq, fb_sq = [], [], []
    for seed in (1, 2, 3):
        mc = np.empty(32 * 32, np.float32)
        ctx.per_bin_monte_carlo(p, spp, seed, mc)
        lrn, _, _, rep = _learned(ctx, scenes.OCCLUDED_SCENE5, params, [0] * 5, [1] * 5, res, spp, seed, steps=800,
                                  cells=0, cells_unbinned=4)
        fb, _, _, rep_fb = _learned(ctx, scenes.OCCLUDED_SCENE5, params, [0] * 5, [1] * 5, res, spp, seed,
                                    steps=800, cells=0, cells_unbinned=4, fallback=1)
        assert rep.fallback_bins == 0 and rep_fb.fallback_bins <= 32 * 32
        mc_sq.append(rmse(mc) ** 2)
        lr_sq.append(rmse(lrn) ** 2)
        fb_sq.append(rmse(fb) ** 2)
    assert np.mean(lr_sq) < 0.9 * np.mean(mc_sq), (lr_sq, mc_sq)
    assert np.mean(fb_sq) < np.mean(lr_sq) * 1.05, (fb_sq, lr_sq)


def test_polynomial_fallback_takes_the_better_bins(ctx):
    """With the polynomial control variate's bins and variances supplied (vcu_control_variates on the
    same problem), bins where the polynomial estimate has the lower variance take it: on the smooth
    sin(8x)e^-y + x^2 + y^2 at 16x16 bins, where crespo2021 is far better than a briefly trained
    network, almost every bin does, and the result is as accurate as the polynomial estimate."""
    res, spp, nb = [16, 16], 64, 256
    exact = scenes.exact_bins(scenes.WAVE2, None, [0, 0], [1, 1], res)[:, 0]
    p = ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], res)
    poly = np.empty(nb, np.float32)
    var = np.empty(nb, np.float32)
    ctx.control_variates(p, _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37), 1023,
                         _lib.CvOpts(spp, 9, 0, 0, 1.0, 0, 0, 0.01, 0, 1.0, 0.0, 0, 0, var.ctypes.data), poly)
    assert np.isfinite(var).all() and (var >= 0).all()
    out, _, st, rep = _learned(ctx, scenes.WAVE2, None, [0, 0], [1, 1], res, spp, 9, steps=50, cells=1, fallback=1,
                               poly=(poly, var))
    assert rep.polynomial_bins >= 0.9 * nb, rep.as_dict()
    took = np.isclose(out, poly, rtol=0, atol=0)
    assert took.sum() == rep.polynomial_bins
    assert scenes.bin_rmse(out, exact[:, None]) <= 1.2 * scenes.bin_rmse(poly, exact[:, None]) + 1e-7


def test_early_stopping_is_deterministic(ctx):
    """Training stops once the held-out error stops improving; the stop and the result are the same
    on a second run (the held-out error is summed in a fixed order)."""
    res, spp = [16, 16], 32
    runs = []
    for _ in range(2):
        out, _, st, rep = _learned(ctx, scenes.WAVE2, None, [0, 0], [1, 1], res, spp, 4, steps=20000, cells=2,
                                   check_every=50)
        runs.append((out, rep.train_steps_run, rep.heldout_mse))
    assert 0 < runs[0][1] < 20000 and runs[0][1] % 50 == 0
    assert np.isfinite(runs[0][2]) and runs[0][2] < 0.05
    assert runs[0][1] == runs[1][1] and runs[0][2] == runs[1][2]
    assert np.array_equal(runs[0][0].view(np.uint32), runs[1][0].view(np.uint32))


def test_invalid_learned_options_are_rejected(ctx):
    p = ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], [4, 4])
    out = np.empty(16, np.float32)
    for opts in (_lib.LearnedOpts(16, 1, 10, 1024, 1e-3, 0, 0, 2, None, 0),        # cells_unbinned 0
                 _lib.LearnedOpts(16, 1, 10, 1024, 1e-3, 0, 0, 40, None, 1),       # 81^2 nodes per bin
                 _lib.LearnedOpts(0, 1, 10, 1024, 1e-3, 0, 0, 2, None, 1)):        # no samples
        with pytest.raises(Exception):
            ctx.learned_control_variates(p, opts, out)
    pb = np.zeros(16, np.float32)
    with pytest.raises(Exception):  # poly_bins without poly_variance
        ctx.learned_control_variates(p, _lib.LearnedOpts(16, 1, 10, 1024, 1e-3, 0, 1, 2, None, 1, 0,
                                                         pb.ctypes.data, None), out)
