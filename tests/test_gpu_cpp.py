"""The C++ drop-in integrators (include/viltrum_cuda.hpp) on the GPU give the C ABI's results.

tests/cpp/dropin.cc is built with the host compiler against libviltrum_cuda.so and run; each of its
outputs is recomputed here through the same library calls (Python binding) and must match bit for
bit: the header adds only the bins(pos) read-in and write-back in viltrum's dim-0-fastest order."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from viltrum_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu


def test_cpp_dropin_matches_c_abi(ctx, tmp_path):
    exe = str(tmp_path / "dropin")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "dropin.cc"), "-L", os.path.join(ROOT, "viltrum_gb300"),
                    "-lviltrum_cuda", "-Wl,-rpath," + os.path.join(ROOT, "viltrum_gb300"), "-o", exe], check=True)
    out = np.array([float(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()],
                   np.float32)
    assert out.size == 256 + 64 + 64 + 16 + 32 + 2 + 64
    img, row, cvb, lrn, glb, bat, cve = np.split(out, [256, 320, 384, 400, 432, 434])
    scene = np.array([2, 1, 0.3, 0.4, 0.05, 0.8, 0.7, 0.6, 0.1, 0.5, 0.5, 0.5, 0.2, 0.25], np.float32)
    # per-bin adaptive nested, 16x16 (image[y][x] flattened = dim-0-fastest bins)
    ref = np.empty(256, np.float32)
    ctx.per_bin_adaptive_nested(ctx.problem(scenes.SCENE2, scene, [0, 0], [1, 1], [16, 16]),
                                _lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37), 15, ref)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    # monte carlo (assign) then monte carlo (accumulate) into the same row
    a = np.empty(64, np.float32)
    b = np.empty(64, np.float32)
    p = ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], [64])
    ctx.per_bin_monte_carlo(p, 256, 7, a)
    ctx.per_bin_monte_carlo_accumulate(p, 256, 9, a)
    assert np.array_equal(row.view(np.uint32), a.view(np.uint32))
    # crespo2021(255 splits, 16 samples, seed 3)
    c = np.empty(64, np.float32)
    ctx.control_variates(ctx.problem(scenes.SCENE2, scene, [0, 0], [1, 1], [64]),
                         _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37), 255, _lib.CvOpts(16, 3, 0, 0, 1.0), c)
    assert np.array_equal(cvb.view(np.uint32), c.view(np.uint32))
    # rr_error_region with cv_fixed_weight(0.5), seed 4
    ctx.control_variates(ctx.problem(scenes.SCENE2, scene, [0, 0], [1, 1], [64]),
                         _lib.Nested(3, 2, 1, 1, 1e-5, 1e-37, 1e-37), 255, _lib.CvOpts(16, 4, 1, 0, 0.5, 2), c)
    assert np.array_equal(cve.view(np.uint32), c.view(np.uint32))
    # learned control variate (16 samples, seed 5, 50 steps, defaults of the header)
    l = np.empty(16, np.float32)
    ctx.learned_control_variates(ctx.problem(scenes.WAVE2, None, [0, 0], [1, 1], [16]),
                                 _lib.LearnedOpts(16, 5, 50, 32768, 3e-3, 0, 1, 2, None, 4), l)
    assert np.array_equal(lrn.view(np.uint32), l.view(np.uint32))
    # adaptive_iterations used directly, then adaptive_tolerance, accumulating into bins that start at 0.5
    gb = np.full(32, 0.5, np.float32)
    ctx.adaptive_iterations_global(ctx.problem(scenes.SCENE2, scene, [0, 0], [1, 1], [32]),
                                   _lib.Nested(3, 2, 0, 0, 1e-5, 1e-37, 1e-37), 127, gb)
    ctx.adaptive_tolerance(ctx.problem(scenes.SCENE2, scene, [0, 0], [1, 1], [32]),
                           _lib.Nested(5, 3, 0, 0, 1e-5, 1e-37, 1e-37), 1e-6, gb)
    assert np.array_equal(glb.view(np.uint32), gb.view(np.uint32))
    # two independent integrals
    hp = np.array([2, 1.5, 0.5, 0, 0, 0, 0, 3.0, 7.0, 0, 0, 0, 0, 0.6, 0.8, 0, 0, 0, 0, 0.9], np.float32)
    items = [dict(dim=2, method=1, budget=100, seed=11, params=hp, rmin=[0, 0], rmax=[1, 1]),
             dict(dim=2, method=0, budget=4096, seed=11, params=hp, rmin=[0, 0], rmax=[1, 1])]
    r, _, _ = ctx.integrate_batch(scenes.HALFSPACE, items, _lib.Nested(3, 2, 0, 0, 1e-5, 1e-37, 1e-37))
    assert np.array_equal(bat.view(np.uint32), r.view(np.uint32))
