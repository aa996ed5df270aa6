"""Shared fixtures.  Tests marked `gpu` need a CUDA device and the built libviltrum_cuda.so;
everything else runs on CPU (the oracle, host logic, library loading and exports)."""
from __future__ import annotations

import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and libviltrum_cuda.so")


@pytest.fixture(scope="session")
def port():
    from oracle import oracle
    return oracle.port()


@pytest.fixture(scope="session")
def ctx():
    from viltrum_gb300 import build
    import viltrum_gb300 as v
    build.build()
    c = v.Context(0)
    yield c
    c.close()


def golden_names(prefix: str = "") -> list[str]:
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, prefix + "*.npz")))


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}
