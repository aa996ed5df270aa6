"""The C-ABI library builds for sm_103a, loads, and exports every entry point include/*.h declares.
No compute call is made here (no GPU is needed)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT
from oracle import oracle as orc


def _declared_symbols() -> set[str]:
    names = set()
    for h in ("viltrum_cuda.h",):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\bint\s+(vcu_\w+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib_path():
    from viltrum_gb300 import build
    return build.build()


def test_library_exports_every_declared_symbol(lib_path):
    declared = _declared_symbols()
    assert {"vcu_create", "vcu_destroy", "vcu_per_bin_monte_carlo", "vcu_per_bin_adaptive_nested"} <= declared
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (vcu_\w+)", out))
    missing = declared - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    lib = ctypes.CDLL(lib_path)
    for name in declared:
        getattr(lib, name)


def test_host_logic_without_device(lib_path):
    """ABI version, channel table, and argument validation that happens before any device use."""
    lib = ctypes.CDLL(lib_path)
    assert lib.vcu_abi_version() == 2
    assert lib.vcu_channels(5) == 1 and lib.vcu_channels(6) == 3 and lib.vcu_channels(99) < 0
    assert lib.vcu_per_bin_monte_carlo(None, None, 1, 1, None, None) == 1  # null context -> INVALID_ARG
    assert lib.vcu_integrate_batch(None, 7, None, None, 0, None, 0, None, None) == 1
    assert lib.vcu_integrate_batch_resident(None, None, 0, None, None) == 1
    assert lib.vcu_per_bin_monte_carlo_accumulate(None, None, 1, 1, None, None, None) == 1
    assert lib.vcu_set_device_memory_limit(None, ctypes.c_uint64(1)) == 1
    assert lib.vcu_destroy(None) == 0


def _compile_dropin(extra, out=None):
    cmd = ["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), *extra,
           os.path.join(ROOT, "tests", "cpp", "dropin.cc")]
    if out:
        cmd += ["-L", os.path.join(ROOT, "viltrum_gb300"), "-lviltrum_cuda", "-o", out]
    else:
        cmd += ["-fsyntax-only"]
    return subprocess.run(cmd, capture_output=True, text=True)


@pytest.mark.skipif(orc.reference_sources() is None, reason="reference sources absent")
def test_cpp_dropin_compiles_against_reference():
    """The CUDA integrators of include/viltrum_cuda.hpp go through the reference's own
    viltrum::integrate(integrator, bins, f, range) (src/integrate.h:72-97) wherever a CPU per-bin
    integrator would: the example compiles against the unmodified reference headers."""
    r = _compile_dropin(["-DWITH_VILTRUM", "-I", orc.reference_sources()])
    assert r.returncode == 0, r.stderr


def test_cpp_dropin_links(lib_path, tmp_path):
    """The standalone form of the example links against libviltrum_cuda.so with the host compiler only."""
    r = _compile_dropin(["-O1"], out=str(tmp_path / "dropin"))
    assert r.returncode == 0, r.stderr


def test_ctypes_structs_match_the_header(tmp_path):
    """Every ctypes mirror in viltrum_gb300/_lib.py has the C struct's size and field offsets (the
    host compiler prints them from include/viltrum_cuda.h)."""
    from viltrum_gb300 import _lib
    pairs = {"vcu_integrand": _lib.Integrand, "vcu_problem": _lib.Problem, "vcu_nested": _lib.Nested, "vcu_stats": _lib.Stats, "vcu_cv": _lib.CvOpts,
             "vcu_learned": _lib.LearnedOpts, "vcu_fubini": _lib.FubiniOpts, "vcu_learned_report": _lib.LearnedReport, "vcu_opts": _lib.Opts,
             "vcu_batch_item": _lib.BatchItem, "vcu_batch_report": _lib.BatchReport}
    lines = ['#include <cstdio>', '#include <cstddef>', '#include "viltrum_cuda.h"', "int main() {"]
    for cname, cls in pairs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.cc"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        c, f, v = ln.split()
        got[(c, f)] = int(v)
    for cname, cls in pairs.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """Without the built CUDA library the Python package raises; nothing falls back to the CPU."""
    from viltrum_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load(str(tmp_path / "libviltrum_cuda.so"))


def test_context_without_device_raises(lib_path):
    """Creating a context where no CUDA device is visible is an error, not a silent CPU run; the
    allocation-free entry point validates its arguments before touching a device."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is visible")
    import viltrum_gb300 as v
    from viltrum_gb300 import _lib
    with pytest.raises(_lib.VcuError):
        v.Context(0)
    lib = ctypes.CDLL(lib_path)
    assert lib.vcu_per_bin_adaptive_nested_static(None, None, ctypes.c_uint64(15), None, None) == 1
