"""integrator_adaptive_tolerance on the GPU (tree built breadth first, leaves added in the reference's
depth-first order) against the reference.  Golden fixtures hold the unmodified reference's bins,
accumulated into a non-zero initial image; larger cases compare with the oracle.  Tolerance: relative
1e-5 per bin against max(|ref|, 1e-3 * max|ref|) (FP32 deterministic Newton-Cotes), and the same
number of leaf regions as the oracle."""
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


@pytest.mark.parametrize("name", golden_names("tolerance_"))
def test_tolerance_matches_reference_golden(ctx, name):
    g = load_golden(name)
    hi, lo, heur, met = [str(x) for x in g["nested"]]
    p = ctx.problem(int(g["kind"]), g["params"], g["rmin"], g["rmax"], g["res"])
    out = np.array(g["initial"], np.float32)
    ctx.adaptive_tolerance(p, _nested(hi, lo, heur, met), float(g["tolerance"]), out)
    ok = _close(out, g["out_bins"].ravel())
    assert ok.all(), int((~ok).sum())


@pytest.mark.parametrize("tol", [1e-5, 1e-7])
def test_tolerance_matches_oracle_scene(ctx, port, tol):
    params = scenes.scene2(7)
    p = ctx.problem(scenes.SCENE2, params, [0, 0], [1, 1], [64, 64])
    out = np.zeros(64 * 64, np.float32)
    st, leaves = ctx.adaptive_tolerance(p, _nested("boole", "simpson", "default", "absolute"), tol, out)
    ref, n = port.adaptive_tolerance(scenes.SCENE2, params, [0, 0], [1, 1], [64, 64], orc.Nested.make(), tol)
    assert leaves == n and st.regions == 2 * n - 1
    assert _close(out, ref[:, 0]).all()


def test_tolerance_capacity_and_python_form(ctx, port):
    params = scenes.scene2(7)
    p = ctx.problem(scenes.SCENE2, params, [0, 0], [1, 1], [16, 16])
    with pytest.raises(_lib.VcuError) as e:
        ctx.adaptive_tolerance(p, _nested("boole", "simpson", "default", "absolute"), 1e-7, np.zeros(256, np.float32),
                               max_regions=101)
    assert e.value.code == 3  # QUEUE_OVERFLOW
    bins = np.full((16, 16), 0.5, np.float32)
    v.integrate(v.integrator_adaptive_tolerance(v.nested(v.boole, v.simpson), 1e-6), bins, v.Integrand.scene2(params),
                v.range_primary(2), ctx=ctx)
    ref, _ = port.adaptive_tolerance(scenes.SCENE2, params, [0, 0], [1, 1], [16, 16], orc.Nested.make(), 1e-6,
                                     initial=np.full(256, 0.5))
    assert _close(bins.transpose(1, 0).ravel(), ref[:, 0]).all()
