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


def test_static_entry_point_status_codes_and_streams(ctx):
    """Status codes of the allocation-free path: a NaN-producing integrand returns
    VCU_NAN_DETECTED and the next clean call returns VCU_OK (the shared status word is cleared per
    call); an unsupported rule pair, heuristic or metric returns VCU_INVALID_ARG, as the regular
    entry point does; a caller's side stream gives the regular entry point's bits."""
    torch = pytest.importorskip("torch")
    fn = _static_fn()
    st = _lib.Nested(3, 2, 0, 0, 1e-5, 1e-37, 1e-37)
    params = scenes.halfspace(3, 2).copy()
    params[1] = np.nan  # a_0 = NaN -> exp(NaN) inside the half-space
    params[19] = 10.0   # the whole domain inside the half-space
    p_nan = ctx.problem(scenes.HALFSPACE, params, [0, 0], [1, 1], [4, 4])
    out = np.empty(16, np.float32)
    assert fn(ctypes.byref(p_nan), ctypes.byref(st), 3, out.ctypes.data, None) == 5
    p_ok = ctx.problem(scenes.SCENE2, scenes.scene2(4), [0, 0], [1, 1], [32, 8])
    regular = np.empty(256, np.float32)
    ctx.per_bin_adaptive_nested(p_ok, _lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37), 15, regular)
    out = np.empty(256, np.float32)
    assert fn(ctypes.byref(p_ok), ctypes.byref(_lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37)), 15,
              out.ctypes.data, None) == 0
    assert np.array_equal(out.view(np.uint32), regular.view(np.uint32))
    for bad in (_lib.Nested(3, 5, 0, 0, 1e-5, 1e-37, 1e-37),   # low rule above the high rule
                _lib.Nested(5, 3, 7, 0, 1e-5, 1e-37, 1e-37),   # unknown heuristic
                _lib.Nested(5, 3, 0, 9, 1e-5, 1e-37, 1e-37)):  # unknown metric
        assert fn(ctypes.byref(p_ok), ctypes.byref(bad), 15, out.ctypes.data, None) == 1
        with pytest.raises(Exception):
            ctx.per_bin_adaptive_nested(p_ok, bad, 15, np.empty(256, np.float32))
    side = torch.cuda.Stream()
    p_dev = ctx.problem(scenes.SCENE2, scenes.scene2(4), [0, 0], [1, 1], [32, 8], mem=_lib.MEM_DEVICE)
    dev = torch.full((256,), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    assert fn(ctypes.byref(p_dev), ctypes.byref(_lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37)), 15, dev.data_ptr(),
              ctypes.c_void_p(side.cuda_stream)) == 0
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), regular.view(np.uint32))


def test_static_entry_point_allocates_nothing(ctx):
    """After one warm-up call, calls of different sizes (host and device bins) leave the device's
    free memory unchanged: the path makes no device allocation."""
    torch = pytest.importorskip("torch")
    fn = _static_fn()
    nested = _lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37)
    dev = torch.empty(128 * 128, dtype=torch.float32, device="cuda")
    host = np.empty(200 * 100, np.float32)
    p_small = ctx.problem(scenes.SCENE2, scenes.scene2(2), [0, 0], [1, 1], [16, 16])
    assert fn(ctypes.byref(p_small), ctypes.byref(nested), 15, host.ctypes.data, None) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for res, mem, buf in (([200, 100], _lib.MEM_HOST, host.ctypes.data), ([128, 128], _lib.MEM_DEVICE, dev.data_ptr()),
                          ([7, 3], _lib.MEM_HOST, host.ctypes.data)):
        p = ctx.problem(scenes.SCENE2, scenes.scene2(2), [0, 0], [1, 1], res, mem=mem)
        assert fn(ctypes.byref(p), ctypes.byref(nested), 15, buf, None) == 0
        torch.cuda.synchronize()
        free, _ = torch.cuda.mem_get_info()
        assert free == free0
