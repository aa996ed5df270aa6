"""Context resources on the GPU: the device-memory limit turns a growth of the context's buffers
past the limit into VCU_OOM -- the allocation-failure path of every entry point -- before anything
is freed or allocated, and the context stays usable afterwards."""
import numpy as np
import pytest

import viltrum_gb300 as v
from viltrum_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu


def test_memory_limit_reports_oom_and_context_recovers():
    ctx = v.Context(0)
    try:
        nested = _lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37)
        small = ctx.problem(scenes.SCENE2, scenes.scene2(7), [0, 0], [1, 1], [64, 64])
        ref = np.empty(64 * 64, np.float32)
        ctx.per_bin_adaptive_nested(small, nested, 15, ref)
        held = ctx.device_memory_held()
        assert held >= 64 * 64 * 4
        # host bins of 512x512 need a 1 MiB staging buffer: past a 256 KiB limit
        ctx.set_device_memory_limit(256 << 10)
        big = ctx.problem(scenes.SCENE2, scenes.scene2(7), [0, 0], [1, 1], [512, 512])
        out = np.empty(512 * 512, np.float32)
        with pytest.raises(v.VcuError) as e:
            ctx.per_bin_adaptive_nested(big, nested, 15, out)
        assert e.value.code == 2 and "memory limit" in str(e.value)
        assert ctx.device_memory_held() == held  # nothing freed, nothing allocated
        # calls that fit keep working under the limit, with identical results
        again = np.empty(64 * 64, np.float32)
        ctx.per_bin_adaptive_nested(small, nested, 15, again)
        assert np.array_equal(again.view(np.uint32), ref.view(np.uint32))
        # other entry points report the same status
        with pytest.raises(v.VcuError) as e:
            ctx.per_bin_monte_carlo(big, 16, 1, out)
        assert e.value.code == 2
        # lifting the limit lets the large call run
        ctx.set_device_memory_limit(0)
        st = ctx.per_bin_adaptive_nested(big, nested, 15, out)
        assert st.flags == 0 and np.isfinite(out).all()
        assert ctx.device_memory_held() >= 512 * 512 * 4
    finally:
        ctx.close()
