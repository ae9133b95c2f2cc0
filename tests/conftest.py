"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on the CPU."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "chebyshev-nonlinear-lab_gb300"
GOLDEN = ROOT / "tests" / "golden"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libnuma_gpu.so")


@pytest.fixture(scope="session")
def oracle():
    """The CPU restatement, single-threaded so that its sums are in a fixed order."""
    from oracle.oracle_lib import Oracle
    o = Oracle()
    o.set_threads(1)
    return o


@pytest.fixture(scope="session")
def ref_counts():
    return json.loads((GOLDEN / "reference_counts.json").read_text())


@pytest.fixture(scope="session")
def ref_small():
    return json.loads((GOLDEN / "reference_small.json").read_text())


@pytest.fixture(scope="session")
def ref_vectors():
    return dict(np.load(GOLDEN / "reference_vectors.npz"))


@pytest.fixture(scope="session")
def c1_rows():
    return json.loads((GOLDEN / "c1_bratu_jacobi.json").read_text())


@pytest.fixture(scope="session")
def lib_path():
    import build  # chebyshev-nonlinear-lab_gb300/build.py
    return build.build()


@pytest.fixture(scope="session")
def gpu(lib_path):
    import numa_gpu
    return numa_gpu.Context(0)


def rel_err(a, b) -> float:
    a, b = np.asarray(a), np.asarray(b)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))
