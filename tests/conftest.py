"""Shared fixtures of the test-suite.

`-m "not gpu"` runs everywhere (oracle vs golden fixtures, host planning, C-ABI
exports); `-m gpu` needs a CUDA device and calls the engine through the C ABI.
"""
from __future__ import annotations

import json
import os
import shutil
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "acceleratedms-osm_gb300"))


# The reference source tree, for the tests that compile its programs against the
# drop-in headers; those tests are skipped unless this variable names the tree.
REFERENCE_ROOT = os.environ.get("MSOSM_REFERENCE_ROOT")


def cuda_compile_flags() -> list[str]:
    """g++ flags for a program that includes cuda_runtime.h and links the CUDA runtime."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    root = Path(nvcc).resolve().parent.parent
    return ["-I", str(root / "include"), "-L", str(root / "lib64"), "-lcudart", f"-Wl,-rpath,{root / 'lib64'}"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def eng():
    """The engine's Python binding; builds the library if it is missing."""
    import pymsosm

    if not pymsosm.LIB_PATH.exists():
        pymsosm.build()
    return pymsosm


@pytest.fixture(scope="session")
def golden_plans():
    return json.loads((GOLDEN / "plan_cases.json").read_text())


@pytest.fixture(scope="session")
def golden_osm():
    return json.loads((GOLDEN / "osm_cases.json").read_text())


@pytest.fixture(scope="session")
def golden_arrays():
    return dict(np.load(GOLDEN / "response.npz"))


def expand_runs(runs, F):
    d = np.full(F, -1, dtype=np.int64)
    for s, n, v in runs:
        d[s:s + n] = v
    return d


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
