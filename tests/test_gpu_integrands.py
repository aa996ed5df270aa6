"""Device and host evaluations of every built-in integrand return the same bits.

This is what makes the GPU's adaptive split decisions comparable one-to-one with the reference
(which runs the same functor on the CPU): the functors use only explicitly rounded operations and
the project's own exp/sin/cos (include/vcu_integrands.h)."""
import numpy as np
import pytest

from viltrum_gb300 import scenes

pytestmark = pytest.mark.gpu

CASES = [
    (scenes.POLY2, None, 2, 0.0, 1.0),
    (scenes.SIN1, None, 1, -30.0, 30.0),
    (scenes.SPHERE3, None, 3, -1.0, 1.0),
    (scenes.WAVE2, None, 2, 0.0, 1.0),
    (scenes.SCENE2, scenes.scene2(7), 2, 0.0, 1.0),
    # one unit bump at the origin: e^(-r^2/2) over r^2/2 in [0, 100], across the clamp at -87
    (scenes.SCENE2, np.array([1, 0, 0, 0, 1, 1], np.float32), 2, 0.0, 10.0),
    (scenes.MOVING_SCENE3, scenes.moving_scene3(7), 3, 0.0, 1.0),
    (scenes.HALFSPACE, scenes.halfspace(11, 4), 4, 0.0, 1.0),
    (scenes.HALFSPACE, scenes.halfspace(12, 6), 6, 0.0, 1.0),
    (scenes.OCCLUDED_SCENE5, scenes.occluded_scene5(7), 5, 0.0, 1.0),
]


@pytest.mark.parametrize("kind,params,dim,lo,hi", CASES)
def test_device_eval_bitwise_equal_host(ctx, port, kind, params, dim, lo, hi):
    rng = np.random.default_rng(kind * 10 + dim)
    x = rng.uniform(lo, hi, size=(20000, dim)).astype(np.float32)
    dev = ctx.eval(kind, params, x)
    host = port.eval(kind, params, x)
    same = dev.view(np.uint32) == host.view(np.uint32)
    assert same.all(), f"{(~same).sum()} of {same.size} values differ; max |diff| " \
                       f"{np.max(np.abs(dev.astype(np.float64) - host)):.3e}"
