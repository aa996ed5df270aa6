"""Per-bin adaptive nested Newton-Cotes: the CUDA path against the reference.

Tolerance (stated by the task for deterministic Newton-Cotes in FP32): relative 1e-5 per bin,
|gpu - ref| <= 1e-5 * max(|ref|, floor) with floor = 1e-3 * max|ref| so that bins whose value is
~0 are judged against the bin-value scale.  The split traces (dimension and float bits of the
popped error of every split) must equal the oracle's in every bin: the device computes the nested
error estimate with the reference's own rounding, so it takes the same decisions, ties included."""
import os

import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle as orc
import viltrum_gb300 as v
from viltrum_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _tol(ref):
    ref = np.asarray(ref, np.float64)
    return RTOL * np.maximum(np.abs(ref), 1e-3 * np.max(np.abs(ref)) + 1e-30)


def _nested(hi, lo, heur, met):
    return _lib.Nested(orc.RULE[hi], orc.RULE[lo], orc.HEUR[heur], orc.METRIC[met], 1e-5, 1e-37, 1e-37)


def _gpu(ctx, kind, params, rmin, rmax, res, nested, iters, trace=False):
    p = ctx.problem(kind, params, rmin, rmax, res)
    nb = int(np.prod(res))
    ch = 3 if kind == scenes.MOVING_SCENE3 else 1
    out = np.empty(nb * ch, np.float32)
    tr = np.empty(nb * iters * 2, np.int32) if trace else None
    st = ctx.per_bin_adaptive_nested(p, nested, iters, out, tr)
    return out.reshape(nb, ch), (tr.reshape(nb, iters, 2) if trace else None), st


@pytest.mark.parametrize("name", golden_names("nc_"))
def test_nested_matches_reference_golden(ctx, name):
    g = load_golden(name)
    hi, lo, heur, met = [str(x) for x in g["nested"]]
    out, _, st = _gpu(ctx, int(g["kind"]), g.get("params"), g["rmin"], g["rmax"], g["res"],
                      _nested(hi, lo, heur, met), int(g["iterations"]))
    ref = g["out_bins"]
    err = np.abs(out.astype(np.float64) - ref)
    assert (err <= _tol(ref)).all(), f"max rel err {np.max(err / np.maximum(np.abs(ref), 1e-30)):.3e}"
    assert st.flags == 0 and st.kernel_launches == 1


@pytest.mark.parametrize("seed,res,rule", [(7, (64, 64), ("boole", "simpson", "default", "absolute")),
                                           (21, (48, 40), ("boole", "simpson", "default", "absolute")),
                                           (5, (32, 32), ("simpson", "trapezoidal", "size", "relative")),
                                           (9, (32, 24), ("boole", "trapezoidal", "default", "relative"))])
def test_nested_scene_against_oracle_with_traces(ctx, port, seed, res, rule):
    params = scenes.scene2(seed)
    iters = 15
    out, gtr, _ = _gpu(ctx, scenes.SCENE2, params, [0, 0], [1, 1], res, _nested(*rule), iters, trace=True)
    ref, otr = port.per_bin_adaptive_nested(scenes.SCENE2, params, [0, 0], [1, 1], res, orc.Nested.make(*rule),
                                            iters, trace=True)
    diff = np.nonzero(~np.all(gtr == otr, axis=(1, 2)))[0]
    assert diff.size == 0, f"{diff.size} bins split differently from the oracle: {diff[:8]}"
    err = np.abs(out.astype(np.float64) - ref)
    bad = np.nonzero(err[:, 0] > _tol(ref)[:, 0])[0]
    assert bad.size == 0, f"{bad.size} bins out of tolerance: {bad[:8]}"


def test_nested_fullsize_matches_oracle(ctx, port):
    """The benchmark workload itself -- 512x512 bins of the 2-D scene (64 Gaussian bumps + 32 disks,
    seed 7), nested(boole, simpson), default absolute heuristic, 15 splits per bin -- against the
    oracle on every bin: identical split traces and bins within 1e-5 relative."""
    params = scenes.scene2(7)
    res = [512, 512]
    nb = 512 * 512
    n = _nested("boole", "simpson", "default", "absolute")
    out, gtr, st = _gpu(ctx, scenes.SCENE2, params, [0, 0], [1, 1], res, n, 15, trace=True)
    assert st.flags == 0
    ref, otr = port.per_bin_adaptive_nested_threads(scenes.SCENE2, params, [0, 0], [1, 1], res, orc.Nested.make(),
                                                    15, 0, nb, os.cpu_count() or 1, trace=True)
    diff = np.nonzero(~np.all(gtr == otr, axis=(1, 2)))[0]
    assert diff.size == 0, f"{diff.size} of {nb} bins split differently from the oracle: {diff[:8]}"
    err = np.abs(out.astype(np.float64) - ref)
    bad = np.nonzero(err[:, 0] > _tol(ref)[:, 0])[0]
    assert bad.size == 0, f"{bad.size} of {nb} bins out of tolerance (max rel {np.max(err / np.abs(ref)):.2e})"


def test_nested_fullsize_scene_properties(ctx):
    """512x512 bins, 16 regions per bin: deterministic, every bin finite, and the result is within
    the quadrature error of the FP64 closed-form bin integrals."""
    params = scenes.scene2(7)
    res = [512, 512]
    n = _nested("boole", "simpson", "default", "absolute")
    a, _, st = _gpu(ctx, scenes.SCENE2, params, [0, 0], [1, 1], res, n, 15)
    b, _, _ = _gpu(ctx, scenes.SCENE2, params, [0, 0], [1, 1], res, n, 15)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.isfinite(a).all() and st.flags == 0
    assert st.evaluations == 512 * 512 * (25 + 15 * 20)
    exact = scenes.exact_bins(scenes.SCENE2, params, [0, 0], [1, 1], res)
    total_err = abs(a.astype(np.float64).sum() - exact.sum()) / exact.sum()
    assert total_err < 1e-3
    rmse = scenes.bin_rmse(a, exact)
    assert rmse < 5e-2


def test_nested_device_buffers_match_host(ctx):
    torch = pytest.importorskip("torch")
    params = scenes.scene2(3)
    res = [64, 32]
    n = _nested("boole", "simpson", "default", "absolute")
    host, _, _ = _gpu(ctx, scenes.SCENE2, params, [0, 0], [1, 1], res, n, 15)
    dev = torch.empty(64 * 32, dtype=torch.float32, device="cuda")
    p = ctx.problem(scenes.SCENE2, params, [0, 0], [1, 1], res, mem=_lib.MEM_DEVICE)
    ctx.per_bin_adaptive_nested(p, n, 15, dev)
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), host.ravel().view(np.uint32))


def test_nested_edge_cases(ctx, port):
    n = _nested("boole", "simpson", "default", "absolute")
    # a single bin, zero splits, odd resolutions, dimbins < dim, 1-D
    for kind, params, rmin, rmax, res, iters in [
        (scenes.POLY2, None, [0, 0], [1, 1], [1], 0),
        (scenes.WAVE2, None, [0, 0], [1, 1], [7, 5], 3),
        (scenes.WAVE2, None, [-1, 2], [3, 2.5], [13], 62),
        (scenes.SIN1, None, [0.0], [3.14159265], [9], 15),
    ]:
        out, _, _ = _gpu(ctx, kind, params, rmin, rmax, res, n, iters)
        ref, _ = port.per_bin_adaptive_nested(kind, params, rmin, rmax, res, orc.Nested.make(), iters)
        assert (np.abs(out.astype(np.float64) - ref) <= _tol(ref)).all()
    # invalid requests are rejected with status codes, not crashes
    with pytest.raises(v.VcuError) as e:
        _gpu(ctx, scenes.POLY2, None, [0, 0], [1, 1], [4], n, 63)
    assert e.value.code == 8
    with pytest.raises(v.VcuError) as e:
        _gpu(ctx, 99, None, [0, 0], [1, 1], [4], n, 3)
    assert e.value.code == 1
    with pytest.raises(v.VcuError) as e:
        _gpu(ctx, scenes.POLY2, None, [0, 0, 0], [1, 1, 1], [4], n, 3)
    assert e.value.code == 1
    with pytest.raises(v.VcuError) as e:
        _gpu(ctx, scenes.SCENE2, np.array([100, 0], np.float32), [0, 0], [1, 1], [4], n, 3)  # > 64 bumps
    assert e.value.code == 1


def test_nested_nan_integrand_is_flagged(ctx):
    params = scenes.halfspace(3, 2).copy()
    params[1] = np.nan  # a_0 = NaN -> exp(NaN) inside the half-space
    params[19] = 10.0   # whole domain inside the half-space
    out, _, st = _gpu(ctx, scenes.HALFSPACE, params, [0, 0], [1, 1], [4, 4],
                      _nested("simpson", "trapezoidal", "default", "absolute"), 3)
    assert st.flags & _lib.FLAG_NAN
    assert np.isnan(out).any()


def test_python_integrate_api(ctx):
    """viltrum-style integrate(integrator, bins, f, range) with the per-bin wrapper's assign semantics."""
    bins = np.full((16, 8), 123.0, np.float32)
    it = v.integrator_per_bin_parallel(v.integrator_adaptive_iterations(
        v.nested(v.boole, v.simpson), v.error_heuristic_default(v.error_metric_absolute()), 15))
    v.integrate(it, bins, v.Integrand.scene2(seed=7), v.range_primary(2), ctx=ctx)
    out, _, _ = _gpu(ctx, scenes.SCENE2, scenes.scene2(7), [0, 0], [1, 1], [16, 8],
                     _nested("boole", "simpson", "default", "absolute"), 15)
    assert np.array_equal(bins, out[:, 0].reshape(8, 16).T)
    one = v.integrate(v.integrator_per_bin_parallel(v.integrator_adaptive_iterations(v.nested(v.boole, v.simpson), 4)),
                      v.Integrand.poly2(), v.range_primary(2), ctx=ctx)
    assert abs(float(one) - 2.0 / 3.0) < 1e-5
