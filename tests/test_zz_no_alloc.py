"""The allocation-free entry point (vcu_per_bin_adaptive_nested_static) returns what the regular
entry point (vcu_per_bin_adaptive_nested) returns, on two calls in a row, through the C ABI.

It exists for callers that may not allocate device memory (plugins inside another allocator's
process, real-time frame loops that cannot take cudaMalloc/cudaFree's device-wide
synchronisation, fixed-budget services): it uses only a scratch array
compiled into the library.  This file is collected last so a failure here does not hide the others;
it passes alone in a fresh process and after the rest of the suite."""
import ctypes

import numpy as np
import pytest

from viltrum_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu


def _static_fn():
    lib = _lib.load()
    fn = lib.vcu_per_bin_adaptive_nested_static
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(_lib.Problem), ctypes.POINTER(_lib.Nested), ctypes.c_uint64, ctypes.c_void_p,
                   ctypes.c_void_p]
    return fn


def test_static_entry_point_matches_regular_one(ctx):
    fn = _static_fn()
    params = scenes.scene2(11)
    res = [96, 80]
    nested = _lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37)
    p = ctx.problem(scenes.SCENE2, params, [0, 0], [1, 1], res)
    regular = np.empty(96 * 80, np.float32)
    ctx.per_bin_adaptive_nested(p, nested, 15, regular)
    for _ in range(2):
        out = np.full(96 * 80, np.nan, np.float32)
        rc = fn(ctypes.byref(p), ctypes.byref(nested), 15, out.ctypes.data, None)
        assert rc == 0
        # same kernel, same inputs: identical bits (well within the 1e-5 relative tolerance)
        assert np.array_equal(out.view(np.uint32), regular.view(np.uint32))


def test_static_entry_point_device_buffers_and_limit(ctx):
    torch = pytest.importorskip("torch")
    fn = _static_fn()
    params = scenes.moving_scene3(5, n_gauss=8, n_disk=8)
    res = [24, 16]
    nested = _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37)
    p_host = ctx.problem(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res)
    regular = np.empty(24 * 16 * 3, np.float32)
    ctx.per_bin_adaptive_nested(p_host, nested, 7, regular)
    p_dev = ctx.problem(scenes.MOVING_SCENE3, params, [0, 0, 0], [1, 1, 1], res, mem=_lib.MEM_DEVICE)
    for _ in range(2):
        dev = torch.full((24 * 16 * 3,), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        rc = fn(ctypes.byref(p_dev), ctypes.byref(nested), 7, dev.data_ptr(), None)
        assert rc == 0
        assert np.array_equal(dev.cpu().numpy().view(np.uint32), regular.view(np.uint32))
    # host-memory bins beyond the compiled-in staging area are rejected before any work
    p_big = ctx.problem(scenes.SCENE2, scenes.scene2(1), [0, 0], [1, 1], [1025, 1024])
    big = np.empty(1025 * 1024, np.float32)
    assert fn(ctypes.byref(p_big), ctypes.byref(_lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37)), 15,
              big.ctypes.data, None) == 8
