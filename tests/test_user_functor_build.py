"""The caller's-own-functor route (include/viltrum_cuda_device.cuh) compiles against the reference's
own viltrum::integrate (src/integrate.h:72-97): tests/cpp/user_functor.cu in its WITH_VILTRUM form
passes the device integrators to viltrum::integrate with user functors -- the std::array form and a
functor of separate floats through viltrum::cuda::device::arity.  nvcc only (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT
from oracle import oracle as orc


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


@pytest.mark.skipif(orc.reference_sources() is None, reason="reference sources absent")
def test_user_functor_unit_compiles_against_reference(tmp_path):
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=compute_103a", "-std=c++17", "--expt-relaxed-constexpr",
           "-DWITH_VILTRUM", "-I", os.path.join(ROOT, "include"), "-I", orc.reference_sources(), "-c",
           os.path.join(ROOT, "tests", "cpp", "user_functor.cu"), "-o", str(tmp_path / "uf.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
