"""A caller's own integrand functors on the GPU through include/viltrum_cuda_device.cuh.

tests/cpp/user_functor.cu is compiled with nvcc for sm_103a and run: it integrates three user
functors -- a 2-D one (the built-in wave written as a user would), a 3-D one taking three floats
(through viltrum::cuda::device::arity), and a 3-channel one -- with the device per-bin adaptive
nested integrators, and prints the bins beside those of the oracle (oracle/oracle_impl.h, the CPU
restatement of the reference, run on the host over the same functors).  Tolerance: 1e-5 relative
per bin (floor 1e-3 of the largest bin), as for the built-in integrands.  The wave's bins, nested
and per-bin Monte Carlo, must also equal the C ABI's built-in wave bit for bit: same kernels,
same arithmetic."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from viltrum_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu


def _close(gpu, ref):
    ref = np.asarray(ref, np.float64)
    tol = 1e-5 * np.maximum(np.abs(ref), 1e-3 * np.max(np.abs(ref)))
    return np.abs(np.asarray(gpu, np.float64) - ref) <= tol


def test_user_functors_match_the_oracle(ctx, tmp_path):
    exe = str(tmp_path / "user_functor")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "--expt-relaxed-constexpr",
                    "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "user_functor.cu"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    vals = {}
    for line in out.splitlines():
        name, n, *rest = line.split()
        vals[name] = np.array([float(x) for x in rest], np.float32)
        assert vals[name].size == int(n)
    for case in ("wave", "shell", "ramp"):
        g, o = vals[case + "_gpu"], vals[case + "_oracle"]
        assert np.isfinite(g).all() and g.size == o.size and o.size > 0
        ok = _close(g, o)
        assert ok.all(), f"{case}: {(~ok).sum()} bins out of tolerance"
    # the user's wave is the built-in one: identical bits through the C ABI
    ref = np.empty(32 * 16, np.float32)
    ctx.per_bin_adaptive_nested(ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], [32, 16]),
                                _lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37), 15, ref)
    assert np.array_equal(vals["wave_gpu"].view(np.uint32), ref.view(np.uint32))
    mc = np.empty(64, np.float32)
    ctx.per_bin_monte_carlo(ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], [64]), 256, 7, mc)
    assert np.array_equal(vals["wave_mc_gpu"].view(np.uint32), mc.view(np.uint32))
