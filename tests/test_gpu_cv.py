"""Control variates + residual Monte Carlo (crespo2021 configuration): the CUDA path against the
reference.

* Region construction is exact: the device builds the same regions in the same heap order as the
  reference (bit-equal ranges).
* The control-variate integral per bin (deterministic) matches the reference's within 1e-5
  relative (floor 1e-3 of the largest bin).
* Replaying the reference's own residual draws (chosen region index + point) gives the reference's
  bins within 1e-5 of the scale of the combined terms (the reference sums its samples in float).
* With Philox draws the estimator's error against the FP64 bin integrals matches the reference
  estimator's at equal samples (mean squared error ratio in [0.7, 1.4] over seeds).
* The importance choices of the residual's region (rr_integral_region, rr_error_region) pass the
  same three checks; their choice probabilities are summed warp-parallel in FP64 rather than in the
  reference's sequential order, far below the 1e-5 tolerance.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle as orc
from test_oracle_golden import cv_strategy
import viltrum_gb300 as v
from viltrum_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu
CRESPO = _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37)


def _gpu_cv(ctx, kind, params, rmin, rmax, res, iters, spp, seed, weight=0, alpha=1.0, replay=None, nested=CRESPO,
            rr=0, sampling=0, mis_power=1.0, mis_cutoff=0.0, rr_factor=0.01):
    p = ctx.problem(kind, params, rmin, rmax, res)
    nb = int(np.prod(res))
    ch = 3 if kind == scenes.MOVING_SCENE3 else 1
    dim = len(rmin)
    out = np.empty(nb * ch, np.float32)
    app = np.empty(nb * ch, np.float32)
    reg = np.empty((iters + 1) * 2 * dim, np.float32)
    rp = None if replay is None else np.ascontiguousarray(replay, np.float32)
    opts = _lib.CvOpts(spp, seed, weight, 0, alpha, rr, sampling, rr_factor, 0, mis_power, mis_cutoff)
    st = ctx.control_variates(p, nested, iters, opts, out, app, reg, rp)
    return out.reshape(nb, ch), app.reshape(nb, ch), reg.reshape(iters + 1, 2, dim), st


@pytest.mark.parametrize("name", golden_names("cv_"))
def test_cv_matches_reference_golden(ctx, port, name):
    g = load_golden(name)
    kind, res, iters, spp, seed = int(g["kind"]), [int(r) for r in g["res"]], int(g["iterations"]), int(g["spp"]), \
        int(g["seed"])
    weight, alpha = int(g["weight"]), float(g["alpha"])
    strategy = cv_strategy(g)
    params = g.get("params")
    ref = port.control_variates(kind, params, g["rmin"], g["rmax"], res,
                                orc.Nested.make("simpson", "trapezoidal", "size", "relative"), iters, spp, seed,
                                weight, alpha, replay=True, approx=True, **strategy)
    # the oracle built on this machine against the fixture (bit for bit where this machine is the one
    # the fixture was made on; NaN payloads and libm's last bits in the pdf samplers' cubic roots are
    # platform-dependent, so elsewhere: the same NaN bins and values within 1e-5 relative)
    gb = g["out_bins"].reshape(-1).astype(np.float64)
    ob = ref["bins"].reshape(-1).astype(np.float64)
    assert np.array_equal(np.isnan(gb), np.isnan(ob))
    gscale = np.abs(np.nan_to_num(gb)) + 1e-3 * np.nanmax(np.abs(gb))
    assert np.all(np.abs(np.nan_to_num(ob - gb)) <= 1e-5 * gscale)
    out, app, reg, st = _gpu_cv(ctx, kind, params, g["rmin"], g["rmax"], res, iters, spp, seed, weight, alpha,
                                replay=ref["replay"], **strategy)
    # 1. the same regions, in the same heap order
    assert np.array_equal(reg.view(np.uint32), g["out_regions"].view(np.uint32))
    # 2. the control-variate integral
    ra = ref["approximation"].astype(np.float64)
    floor = 1e-3 * np.max(np.abs(ra))
    assert np.all(np.abs(app - ra) <= 1e-5 * np.maximum(np.abs(ra), floor))
    # 3. the residual estimator on the reference's own draws (the pdf samplers give NaN where the
    #    reference does: a region whose nodes are all 0 has the pdf 0/0)
    rb = g["out_bins"].astype(np.float64)
    nan = np.isnan(rb)
    assert np.array_equal(np.isnan(out), nan)
    scale = np.abs(rb) + np.abs(ra) + floor
    err = np.where(nan, 0.0, np.abs(out - rb))
    assert np.all(err <= 1e-5 * np.where(nan, 1.0, scale)), f"max scaled err {np.nanmax(err / scale):.3e}"
    assert st.flags == (_lib.FLAG_NAN if nan.any() else 0)


def test_cv_statistics_against_fp64(ctx, port):
    params = scenes.moving_scene3(7, n_gauss=16, n_disk=16)
    res, iters, spp = [32, 32], 511, 16
    exact = scenes.exact_bins(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res, t_nodes=96)
    gpu_sq, ref_sq = [], []
    for seed in (1, 2, 3, 4):
        out, app, _, _ = _gpu_cv(ctx, scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res, iters, spp, seed)
        gpu_sq.append(np.mean((out - exact) ** 2))
        ref = port.control_variates(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res,
                                    orc.Nested.make("simpson", "trapezoidal", "size", "relative"), iters, spp, seed)
        ref_sq.append(np.mean((ref["bins"] - exact) ** 2))
    ratio = np.mean(gpu_sq) / np.mean(ref_sq)
    assert 0.7 <= ratio <= 1.4, (gpu_sq, ref_sq)


def test_cv_occluded_scene_statistics(ctx, port):
    """The 5-D occluded scene, whose residual evaluates its drawn points two at a time with the scene's
    terms culled to the bin (pair_culled): with Philox draws its error against a plain Monte Carlo
    truth (2^16 samples per bin) matches the oracle's control variates' at equal samples."""
    params = scenes.occluded_scene5(7)
    lo, hi = [0] * 5, [1] * 5
    res, iters, spp = [16, 16], 255, 64
    p = ctx.problem(scenes.OCCLUDED_SCENE5, params, lo, hi, res)
    truth = np.empty(16 * 16, np.float32)
    ctx.per_bin_monte_carlo(p, 1 << 16, 99, truth)
    truth = truth.astype(np.float64)
    gpu_sq, ref_sq = [], []
    for seed in (1, 2, 3, 4):
        out, _, _, st = _gpu_cv(ctx, scenes.OCCLUDED_SCENE5, params, lo, hi, res, iters, spp, seed)
        assert st.flags == 0
        gpu_sq.append(np.mean((out[:, 0] - truth) ** 2))
        ref = port.control_variates(scenes.OCCLUDED_SCENE5, params, lo, hi, res,
                                    orc.Nested.make("simpson", "trapezoidal", "size", "relative"), iters, spp, seed)
        ref_sq.append(np.mean((ref["bins"].ravel() - truth) ** 2))
    ratio = np.mean(gpu_sq) / np.mean(ref_sq)
    assert 0.6 <= ratio <= 1.6, (gpu_sq, ref_sq)


def test_cv_fullsize_matches_oracle(ctx, port):
    """The control-variate workload at its full size -- integrator_crespo2021(2^14 - 1 splits, 64
    residual samples) on the RGB moving-disk scene into 512x512 bins -- against the oracle: the same
    2^14 regions in the same heap order (bit-equal ranges), the control-variate integral within 1e-5
    relative in every bin and channel, and, replaying the oracle's own residual draws for every bin,
    the oracle's bins within 1e-5 of the scale of the combined terms."""
    params = scenes.moving_scene3(7)
    res, iters, spp, seed = [512, 512], (1 << 14) - 1, 64, 3
    ref = port.control_variates(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res,
                                orc.Nested.make("simpson", "trapezoidal", "size", "relative"), iters, spp, seed,
                                regions=True, replay=True, approx=True)
    out, app, reg, st = _gpu_cv(ctx, scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res, iters, spp, seed,
                                replay=ref["replay"])
    assert st.flags == 0
    assert np.array_equal(reg.view(np.uint32), ref["regions"].view(np.uint32))
    ra = ref["approximation"].astype(np.float64)
    floor = 1e-3 * np.max(np.abs(ra))
    aerr = np.abs(app - ra)
    assert np.all(aerr <= 1e-5 * np.maximum(np.abs(ra), floor)), \
        f"max rel approximation err {np.max(aerr / np.maximum(np.abs(ra), floor)):.3e}"
    rb = ref["bins"].astype(np.float64)
    scale = np.abs(rb) + np.abs(ra) + floor
    err = np.abs(out - rb)
    assert np.all(err <= 1e-5 * scale), f"max scaled err {np.max(err / scale):.3e}"


def test_cv_fullsize_crespo(ctx):
    """The same workload with the device's Philox draws: deterministic, finite, regions tiling the
    domain, and far more accurate than plain Monte Carlo at the same samples."""
    params = scenes.moving_scene3(7)
    res = [512, 512]
    a, app, reg, st = _gpu_cv(ctx, scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res, (1 << 14) - 1, 64, 3)
    b, _, _, _ = _gpu_cv(ctx, scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res, (1 << 14) - 1, 64, 3)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.isfinite(a).all() and st.flags == 0
    # regions tile the domain: their volumes sum to 1
    vol = np.prod(reg[:, 1, :].astype(np.float64) - reg[:, 0, :], axis=1)
    assert abs(vol.sum() - 1.0) < 1e-6
    exact = scenes.exact_bins(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res, t_nodes=64)
    rmse_cv = scenes.bin_rmse(a, exact)
    p = ctx.problem(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res)
    mc = np.empty(512 * 512 * 3, np.float32)
    ctx.per_bin_monte_carlo(p, 64, 3, mc)
    rmse_mc = scenes.bin_rmse(mc.reshape(-1, 3), exact)
    assert rmse_cv < 0.5 * rmse_mc, (rmse_cv, rmse_mc)


def test_python_crespo2021_api(ctx):
    bins = np.zeros((16, 16, 3), np.float32)
    params = scenes.moving_scene3(7, n_gauss=8, n_disk=8)
    v.integrate(v.integrator_crespo2021(255, 16, 3), bins, v.Integrand.moving_scene3(params), v.range_primary(3),
                ctx=ctx)
    out, _, _, _ = _gpu_cv(ctx, scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], [16, 16], 255, 16, 3)
    assert np.array_equal(bins.transpose(1, 0, 2).reshape(-1, 3), out)


@pytest.mark.parametrize("rr", [orc.RR_INTEGRAL, orc.RR_ERROR])
def test_cv_importance_many_regions_per_bin(ctx, port, rr):
    """Bins holding hundreds of regions (the choice tables span many warp-wide chunks), replaying
    the oracle's draws: the same bins within 1e-5 of the scale of the combined terms."""
    params = scenes.scene2(7, n_gauss=16, n_disk=8)
    res, iters, spp = [2, 2], 2047, 96
    nst = orc.Nested.make("simpson", "trapezoidal", "size", "relative")
    ref = port.control_variates(scenes.SCENE2, params, [0, 0], [1, 1], res, nst, iters, spp, 5, replay=True,
                                approx=True, rr=rr)
    assert ref["replay"][:, :, 0].max() > 300  # region indices deep into the lists
    out, app, _, st = _gpu_cv(ctx, scenes.SCENE2, params, [0, 0], [1, 1], res, iters, spp, 5, replay=ref["replay"],
                              rr=rr)
    ra = ref["approximation"].astype(np.float64)
    rb = ref["bins"].astype(np.float64)
    scale = np.abs(rb) + np.abs(ra) + 1e-3 * np.max(np.abs(ra))
    assert np.all(np.abs(out - rb) <= 1e-5 * scale), np.max(np.abs(out - rb) / scale)
    assert st.flags == 0


@pytest.mark.parametrize("rr", [orc.RR_INTEGRAL, orc.RR_ERROR])
def test_cv_importance_statistics_against_fp64(ctx, port, rr):
    """Philox importance choice: mean squared error against the FP64 bin integrals comparable to the
    reference estimator's (std::mt19937 draws) over four seeds, for the optimised weight and for
    alpha = 0 (plain Monte Carlo whose points are importance-sampled among the regions)."""
    params = scenes.moving_scene3(7, n_gauss=16, n_disk=16)
    res, iters, spp = [32, 32], 511, 16
    exact = scenes.exact_bins(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res, t_nodes=96)
    nst = orc.Nested.make("simpson", "trapezoidal", "size", "relative")
    for weight, alpha in ((0, 1.0), (1, 0.0)):
        gpu_sq, ref_sq = [], []
        for seed in (1, 2, 3, 4):
            out, _, _, st = _gpu_cv(ctx, scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res, iters, spp, seed,
                                    weight, alpha, rr=rr)
            assert st.flags == 0
            gpu_sq.append(np.mean((out - exact) ** 2))
            ref = port.control_variates(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res, nst, iters, spp,
                                        seed, weight, alpha, rr=rr)
            ref_sq.append(np.mean((ref["bins"] - exact) ** 2))
        ratio = np.mean(gpu_sq) / np.mean(ref_sq)
        assert 0.7 <= ratio <= 1.4, (weight, gpu_sq, ref_sq)


def test_cv_importance_python_api_and_bad_choice(ctx):
    params = scenes.scene2(7, n_gauss=8, n_disk=4)
    bins = np.zeros((8, 8), np.float32)
    integ = v.integrator_adaptive_variance_reduction_parallel(
        v.nested(v.simpson, v.trapezoidal), v.error_heuristic_size(v.error_metric_relative(), 1e-5), 127,
        v.rr_error_region(), v.cv_optimize_weight(), 16, 9)
    v.integrate(integ, bins, v.Integrand.scene2(params), v.range_primary(2), ctx=ctx)
    out, _, _, _ = _gpu_cv(ctx, scenes.SCENE2, params, [0, 0], [1, 1], [8, 8], 127, 16, 9, rr=orc.RR_ERROR)
    assert np.array_equal(bins.T.reshape(-1), out[:, 0])
    p = ctx.problem(scenes.SCENE2, params, [0, 0], [1, 1], [8, 8])
    o = np.empty(64, np.float32)
    for bad in (_lib.CvOpts(4, 1, 0, 0, 1.0, 4), _lib.CvOpts(4, 1, 0, 0, 1.0, 1, 4),
                _lib.CvOpts(4, 1, 0, 0, 1.0, 1, 0, 0.01, 1)):
        with pytest.raises(_lib.VcuError) as e:
            ctx.control_variates(p, CRESPO, 15, bad, o)
        assert e.value.code == 1
    # the pdf exists for Simpson's rule only
    boole = _lib.Nested(5, 3, 1, 1, 1e-5, 1e-37, 1e-37)
    for bad in (_lib.CvOpts(4, 1, 0, 0, 1.0, 3), _lib.CvOpts(4, 1, 0, 0, 1.0, 0, 1)):
        with pytest.raises(_lib.VcuError) as e:
            ctx.control_variates(p, boole, 15, bad, o)
        assert e.value.code == 8


PDF_STRATEGIES = [  # (rr, sampling, mis power, mis cutoff)
    (orc.RR_PDF, orc.RS_UNIFORM, 1.0, 0.0), (orc.RR_UNIFORM, orc.RS_IMPORTANCE, 1.0, 0.0),
    (orc.RR_PDF, orc.RS_IMPORTANCE, 1.0, 0.0), (orc.RR_PDF, orc.RS_RUSSIAN_ROULETTE, 1.0, 0.0),
    (orc.RR_UNIFORM, orc.RS_MIS, 1.0, 0.0), (orc.RR_PDF, orc.RS_MIS, 2.0, 0.05)]


@pytest.mark.parametrize("rr,sampling,power,cutoff", PDF_STRATEGIES)
def test_cv_pdf_strategies_replay_3d(ctx, port, rr, sampling, power, cutoff):
    """The Simpson pdf in three dimensions (prod_d exp(-a x) cos(b x) over the whole cube: the
    half-space holds it all, so no region is all zero and no pdf is 0/0): the oracle's draws
    replayed give its bins within 1e-5 of the scale."""
    params = np.array([3, 0.5, 1.0, 0.3, 0, 0, 0, 2.0, 3.0, 1.5, 0, 0, 0, 0.2, 0.3, 0.1, 0, 0, 0, 10.0], np.float32)
    res, iters, spp = [8, 8], 255, 16
    nst = orc.Nested.make("simpson", "trapezoidal", "size", "relative")
    kw = dict(rr=rr, sampling=sampling, mis_power=power, mis_cutoff=cutoff)
    ref = port.control_variates(scenes.HALFSPACE, params, [0, 0, 0], [1, 1, 1], res, nst, iters, spp, 7, replay=True,
                                approx=True, **kw)
    out, _, _, st = _gpu_cv(ctx, scenes.HALFSPACE, params, [0, 0, 0], [1, 1, 1], res, iters, spp, 7,
                            replay=ref["replay"], **kw)
    ra = ref["approximation"].astype(np.float64)
    rb = ref["bins"].astype(np.float64)
    assert np.isfinite(rb).all()
    scale = np.abs(rb) + np.abs(ra) + 1e-3 * np.max(np.abs(ra))
    assert np.all(np.abs(out - rb) <= 1e-5 * scale), np.max(np.abs(out - rb) / scale)
    assert st.flags == 0


@pytest.mark.parametrize("rr,sampling,power,cutoff", PDF_STRATEGIES)
def test_cv_pdf_strategies_statistics_against_fp64(ctx, port, rr, sampling, power, cutoff):
    """Philox draws through the device's own inverse cdf: the mean squared error against the FP64
    bin integrals comparable to the reference estimator's over eight seeds, with the plain
    Monte Carlo weight (alpha = 0) so that the pdf's weights carry the whole estimate (wave2, whose
    regions are never all zero)."""
    res, iters, spp = [64, 64], 1023, 16
    exact = scenes.exact_bins(scenes.WAVE2, None, [0, 0], [1, 1], res)
    nst = orc.Nested.make("simpson", "trapezoidal", "size", "relative")
    kw = dict(rr=rr, sampling=sampling, mis_power=power, mis_cutoff=cutoff)
    gpu_sq, ref_sq = [], []
    for seed in range(1, 9):
        out, _, _, st = _gpu_cv(ctx, scenes.WAVE2, None, [0, 0], [1, 1], res, iters, spp, seed, 1, 0.0, **kw)
        assert np.isfinite(out).all() and st.flags == 0
        gpu_sq.append(np.mean((out - exact) ** 2))
        ref = port.control_variates(scenes.WAVE2, None, [0, 0], [1, 1], res, nst, iters, spp, seed, 1, 0.0, **kw)
        ref_sq.append(np.mean((ref["bins"] - exact) ** 2))
    ratio = np.mean(gpu_sq) / np.mean(ref_sq)
    assert 0.7 <= ratio <= 1.4, (gpu_sq, ref_sq)


def test_cv_fubini_tail_against_reference_statistics(ctx):
    """integrator_crespo2021_infinite<2> over the moving-disk scene (regions over x, y; time by Monte
    Carlo in every evaluation): the reference draws its tail samples from one sequential stream, so
    its outputs for eight seeds (fixture) are compared statistically -- the device's mean squared
    error against the FP64 truth over the same seeds within [0.7, 1.4] of the reference's."""
    g = load_golden("fubini_moving3_rgb_bins32x32_it511_mc8_spp16")
    params, res = g["params"], [int(r) for r in g["res"]]
    exact = scenes.exact_bins(scenes.MOVING_SCENE3, params, g["rmin"], g["rmax"], res, t_nodes=96)
    ref_sq = [np.mean((b - exact) ** 2) for b in g["out_bins"]]
    p = ctx.problem(scenes.MOVING_SCENE3, params, g["rmin"], g["rmax"], res)
    gpu_sq = []
    reg = np.empty((int(g["iterations"]) + 1) * 2 * 2, np.float32)
    for seed in g["seeds"]:
        out = np.empty(int(np.prod(res)) * 3, np.float32)
        opts = _lib.CvOpts(int(g["spp"]), int(seed), 0, 0, 1.0, 0, 0, 0.01, 0, 1.0, 0.0, 2, int(g["mc_samples"]))
        st = ctx.control_variates(p, CRESPO, int(g["iterations"]), opts, out, None, reg)
        assert st.flags == 0 and np.isfinite(out).all()
        gpu_sq.append(np.mean((out.reshape(-1, 3) - exact) ** 2))
        # the regions tile the (x, y) square
        r = reg.reshape(-1, 2, 2).astype(np.float64)
        assert abs(np.prod(r[:, 1] - r[:, 0], axis=1).sum() - 1.0) < 1e-6
    ratio = np.mean(gpu_sq) / np.mean(ref_sq)
    assert 0.7 <= ratio <= 1.4, (gpu_sq, ref_sq)


def test_cv_fubini_python_api_and_limits(ctx):
    params = scenes.moving_scene3(7, n_gauss=8, n_disk=8)
    bins = np.zeros((16, 16, 3), np.float32)
    v.integrate(v.integrator_crespo2021_infinite(2, 255, 4, 16, 3), bins, v.Integrand.moving_scene3(params),
                v.range_primary(3), ctx=ctx)
    p = ctx.problem(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], [16, 16])
    out = np.empty(16 * 16 * 3, np.float32)
    ctx.control_variates(p, CRESPO, 255, _lib.CvOpts(16, 3, 0, 0, 1.0, 0, 0, 0.01, 0, 1.0, 0.0, 2, 4), out)
    assert np.array_equal(bins.transpose(1, 0, 2).reshape(-1), out)
    # a deterministic function of its inputs: the same call gives the same bits
    again = np.empty_like(out)
    ctx.control_variates(p, CRESPO, 255, _lib.CvOpts(16, 3, 0, 0, 1.0, 0, 0, 0.01, 0, 1.0, 0.0, 2, 4), again)
    assert np.array_equal(out.view(np.uint32), again.view(np.uint32))
    # regions over 2 of >= 3 dimensions, nested(simpson, trapezoidal), at least one tail sample
    q = ctx.problem(scenes.SCENE2, scenes.scene2(7), [0, 0], [1, 1], [8, 8])
    bad = [(q, CRESPO, _lib.CvOpts(4, 1, 0, 0, 1.0, 0, 0, 0.01, 0, 1.0, 0.0, 2, 4), 8),
           (p, CRESPO, _lib.CvOpts(4, 1, 0, 0, 1.0, 0, 0, 0.01, 0, 1.0, 0.0, 1, 4), 8),
           (p, CRESPO, _lib.CvOpts(4, 1, 0, 0, 1.0, 0, 0, 0.01, 0, 1.0, 0.0, 2, 0), 1),
           (p, _lib.Nested(5, 3, 1, 1, 1e-5, 1e-37, 1e-37), _lib.CvOpts(4, 1, 0, 0, 1.0, 0, 0, 0.01, 0, 1.0, 0.0, 2, 4), 8)]
    for prob, nst, opts, code in bad:
        with pytest.raises(_lib.VcuError) as e:
            ctx.control_variates(prob, nst, 15, opts, np.empty(16 * 16 * 3, np.float32))
        assert e.value.code == code


def test_walk_unbounded_dimension_against_reference_statistics(ctx):
    """The random walk over the scene, an integrand of unbounded dimension over range_infinite:
    fixtures hold the unmodified reference's per-bin Monte Carlo and crespo2021_infinite<2> bins for
    eight seeds each.  Truth: the device's per-bin Monte Carlo with 2^16 walks per bin.  The
    reference's seed mean lies within 4 standard errors of it in all but a few bins (the device's walk
    has the reference's expectation), and over the same seeds the device's mean squared error for both
    integrators is within [0.7, 1.4] of the reference's."""
    gm = load_golden("walk_mc_bins16x16_spp256")
    gc = load_golden("walk_crespo_infinite_bins16x16_it255_mc8_spp16")
    params, res = gm["params"], [16, 16]
    p = ctx.problem(scenes.WALK2, params, [0, 0], [1, 1], res)
    truth = np.empty(256, np.float32)
    ctx.per_bin_monte_carlo(p, 1 << 16, 99, truth)
    truth = truth.astype(np.float64)
    ref = gm["out_bins"].astype(np.float64)
    se = ref.std(axis=0, ddof=1) / np.sqrt(ref.shape[0])
    assert int((np.abs(ref.mean(axis=0) - truth) > 4 * se + 1e-6).sum()) <= 3
    for g, run in ((gm, lambda s, o: ctx.per_bin_monte_carlo(p, int(gm["spp"]), s, o)),
                   (gc, lambda s, o: ctx.control_variates(
                       p, CRESPO, int(gc["iterations"]),
                       _lib.CvOpts(int(gc["spp"]), s, 0, 0, 1.0, 0, 0, 0.01, 0, 1.0, 0.0, 2, int(gc["mc_samples"])), o))):
        gpu_sq, ref_sq = [], []
        for i, seed in enumerate(g["seeds"]):
            out = np.empty(256, np.float32)
            run(int(seed), out)
            gpu_sq.append(np.mean((out - truth) ** 2))
            ref_sq.append(np.mean((g["out_bins"][i] - truth) ** 2))
        ratio = np.mean(gpu_sq) / np.mean(ref_sq)
        assert 0.7 <= ratio <= 1.4, (str(g["method"]), gpu_sq, ref_sq)


def test_walk_python_api(ctx):
    bins = np.zeros((8, 8), np.float32)
    v.integrate(v.integrator_per_bin_parallel(v.monte_carlo(64, 3)), bins, v.Integrand.walk2(),
                v.range_infinite([0, 0], [1, 1]), ctx=ctx)
    assert np.isfinite(bins).all() and bins.mean() > 0
    c = np.zeros((8, 8), np.float32)
    v.integrate(v.integrator_crespo2021_infinite(2, 127, 4, 8, 3), c, v.Integrand.walk2(),
                v.range_infinite([0, 0], [1, 1]), ctx=ctx)
    assert np.isfinite(c).all() and abs(c.mean() - bins.mean()) < 0.2 * bins.mean()
