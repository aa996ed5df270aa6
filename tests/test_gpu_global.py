"""integrator_adaptive_iterations used directly (one heap over the whole range, regions added into
the bins) on the GPU against the reference.

The golden fixtures hold the unmodified reference's bins, accumulated into a non-zero initial image.
Tolerance: relative 1e-5 per bin against max(|ref|, 1e-3 * max|ref|) (FP32 deterministic
Newton-Cotes); the region set itself is the control-variate generator's, whose split sequence is
bit-identical to the reference's."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle as orc
import viltrum_gb300 as v
from viltrum_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu


def _nested(hi, lo, heur, met):
    return _lib.Nested(orc.RULE[hi], orc.RULE[lo], orc.HEUR[heur], orc.METRIC[met], 1e-5, 1e-37, 1e-37)


def _close(gpu, ref):
    ref = np.asarray(ref, np.float64)
    tol = 1e-5 * np.maximum(np.abs(ref), 1e-3 * np.max(np.abs(ref)) + 1e-30)
    return np.abs(np.asarray(gpu, np.float64) - ref) <= tol


@pytest.mark.parametrize("name", golden_names("global_"))
def test_global_matches_reference_golden(ctx, name):
    g = load_golden(name)
    hi, lo, heur, met = [str(x) for x in g["nested"]]
    p = ctx.problem(int(g["kind"]), g["params"], g["rmin"], g["rmax"], g["res"])
    out = np.array(g["initial"], np.float32)
    st = ctx.adaptive_iterations_global(p, _nested(hi, lo, heur, met), int(g["iterations"]), out)
    ref = g["out_bins"].ravel()
    ok = _close(out, ref)
    assert ok.all(), (int((~ok).sum()), float(np.max(np.abs(out - ref))))
    assert st.regions == int(g["iterations"]) + 1


def test_global_matches_oracle_larger(ctx, port):
    """64x64 bins, 4095 splits, boole over trapezoidal."""
    params = scenes.scene2(7)
    p = ctx.problem(scenes.SCENE2, params, [0, 0], [1, 1], [64, 64])
    out = np.zeros(64 * 64, np.float32)
    ctx.adaptive_iterations_global(p, _nested("boole", "trapezoidal", "default", "absolute"), 4095, out)
    ref = port.adaptive_global(scenes.SCENE2, params, [0, 0], [1, 1], [64, 64],
                               orc.Nested.make("boole", "trapezoidal"), 4095)[:, 0]
    assert _close(out, ref).all()


def test_global_python_forms(ctx, port):
    """integrate(integrator_adaptive_iterations(...), bins, f, range) accumulates into a 2-D array, and
    the single-value form equals the reference's integrate(I, f, range)."""
    params = scenes.halfspace(3, 3)
    bins = np.full((8, 4), 0.25, np.float32)  # resolution (8, 4): dim 0 has 8 bins
    integ = v.integrator_adaptive_iterations(v.nested(v.simpson, v.trapezoidal), 200)
    v.integrate(integ, bins, v.Integrand.halfspace(params), v.range_primary(3), ctx=ctx)
    ref = port.adaptive_global(scenes.HALFSPACE, params, [0] * 3, [1] * 3, [8, 4],
                               orc.Nested.make("simpson", "trapezoidal"), 200, initial=np.full(32, 0.25))[:, 0]
    flat = bins.transpose(1, 0).ravel()  # viltrum's linear order: dim 0 fastest
    assert _close(flat, ref).all()
    single = v.integrate(integ, v.Integrand.halfspace(params), v.range_primary(3), ctx=ctx)
    ref1 = port.integrate_single(scenes.HALFSPACE, params, [0] * 3, [1] * 3, 1, 201, 0,
                                 orc.Nested.make("simpson", "trapezoidal"))
    assert abs(float(single) - ref1) <= 1e-5 * abs(ref1) + 1e-12
