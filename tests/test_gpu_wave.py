"""The adaptive heap's regions built in parallel waves equal the sequential generator's.

Both generators serve vcu_control_variates and vcu_adaptive_iterations_global
(VCU_CV_GENERATOR=wave|sequential selects one; by default the waves run from 128 splits on).  The
waves split, together, the regions of largest bottleneck error, and the host replays the
reference's heap sequence on their errors; the result must be the sequential generator's region for
region and position for position -- bit-equal region ranges in heap order and bit-equal bins (the
control variates' per-bin lists and residual draws depend on that order)."""
import os

import numpy as np
import pytest

from conftest import golden_names, load_golden
from viltrum_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu

ST_SIZE_REL = _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37)
ST_ABS = _lib.Nested(3, 2, 0, 0, 1e-5, 1e-37, 1e-37)
BS_REL = _lib.Nested(5, 3, 0, 1, 1e-5, 1e-37, 1e-37)
BT_ABS = _lib.Nested(5, 2, 0, 0, 1e-5, 1e-37, 1e-37)


def _with(generator, fn):
    os.environ["VCU_CV_GENERATOR"] = generator
    try:
        return fn()
    finally:
        del os.environ["VCU_CV_GENERATOR"]


def _cv(ctx, kind, params, rmin, rmax, res, nested, iters, spp, opts_extra=(), rdim=None):
    p = ctx.problem(kind, params, rmin, rmax, res)
    ch = 3 if kind == scenes.MOVING_SCENE3 else 1
    rdim = rdim or len(rmin)

    def run():
        out = np.empty(int(np.prod(res)) * ch, np.float32)
        reg = np.empty((iters + 1) * 2 * rdim, np.float32)
        st = ctx.control_variates(p, nested, iters, _lib.CvOpts(spp, 5, 0, 0, 1.0, *opts_extra), out, None, reg)
        return out, reg, st
    return run


CASES = [
    ("moving3_rgb_crespo", scenes.MOVING_SCENE3, scenes.moving_scene3(7, n_gauss=16, n_disk=16), 3, [32, 32],
     ST_SIZE_REL, 4095),
    ("scene2_abs", scenes.SCENE2, scenes.scene2(7), 2, [64, 64], ST_ABS, 4095),
    ("halfspace3_boole_rel", scenes.HALFSPACE, scenes.halfspace(3, 3), 3, [16, 16], BS_REL, 1023),
    ("occluded5", scenes.OCCLUDED_SCENE5, scenes.occluded_scene5(7), 5, [16, 16], ST_SIZE_REL, 1023),
    ("scene2_boole_trap", scenes.SCENE2, scenes.scene2(9, n_gauss=8, n_disk=4), 2, [32, 32], BT_ABS, 2047),
]


@pytest.mark.parametrize("name,kind,params,dim,res,nested,iters", CASES, ids=[c[0] for c in CASES])
def test_wave_generator_equals_sequential(ctx, name, kind, params, dim, res, nested, iters):
    run = _cv(ctx, kind, params, [0] * dim, [1] * dim, res, nested, iters, 8)
    a_out, a_reg, a_st = _with("sequential", run)
    b_out, b_reg, b_st = _with("wave", run)
    assert np.array_equal(a_reg.view(np.uint32), b_reg.view(np.uint32))
    assert np.array_equal(a_out.view(np.uint32), b_out.view(np.uint32))
    assert a_st.regions == b_st.regions == iters + 1


def test_wave_generator_fubini_and_global(ctx):
    params = scenes.moving_scene3(7, n_gauss=16, n_disk=16)
    run = _cv(ctx, scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], [32, 32], ST_SIZE_REL, 2047, 8,
              (0, 0, 0.01, 0, 1.0, 0.0, 2, 4), rdim=2)
    a_out, a_reg, _ = _with("sequential", run)
    b_out, b_reg, _ = _with("wave", run)
    assert np.array_equal(a_reg.view(np.uint32), b_reg.view(np.uint32))
    assert np.array_equal(a_out.view(np.uint32), b_out.view(np.uint32))
    # integrator_adaptive_iterations used directly: one heap over the range, accumulating
    p = ctx.problem(scenes.SCENE2, scenes.scene2(7), [0, 0], [1, 1], [128, 128])

    def glob():
        b = np.full(128 * 128, 0.5, np.float32)
        ctx.adaptive_iterations_global(p, BT_ABS, 8191, b)
        return b
    assert np.array_equal(_with("sequential", glob).view(np.uint32), _with("wave", glob).view(np.uint32))


def test_wave_generator_ties_fall_back(ctx):
    """One bump and one disk on an empty square: most regions have error exactly 0, so the split
    set is decided among thousands of equal errors; the waves either replay it or give up and the
    sequential generator builds it -- the result is the same either way."""
    params = scenes.scene2(3, n_gauss=1, n_disk=1)
    run = _cv(ctx, scenes.SCENE2, params, [0, 0], [1, 1], [32, 32], ST_ABS, 3000, 4)
    a_out, a_reg, _ = _with("sequential", run)
    b_out, b_reg, _ = _with("wave", run)
    assert np.array_equal(a_reg.view(np.uint32), b_reg.view(np.uint32))
    assert np.array_equal(a_out.view(np.uint32), b_out.view(np.uint32))


@pytest.mark.parametrize("name", golden_names("cv_"))
def test_wave_generator_reference_regions(ctx, name):
    """The reference's own region sets (golden fixtures), built by the waves."""
    g = load_golden(name)
    if "sampling" in g or "rr" in g:
        pytest.skip("same regions as the uniform fixtures: the strategies change the residual only")
    dim = len(g["rmin"])
    run = _cv(ctx, int(g["kind"]), g.get("params"), g["rmin"], g["rmax"], [int(r) for r in g["res"]], ST_SIZE_REL,
              int(g["iterations"]), int(g["spp"]))
    _, reg, _ = _with("wave", run)
    assert np.array_equal(reg.reshape(-1, 2, dim).view(np.uint32), g["out_regions"].view(np.uint32))
