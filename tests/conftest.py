"""Shared fixtures.  `-m "not gpu"` runs on any host; `-m gpu` needs a CUDA device
and the in-tree library built by ``__graft_entry__.build()``."""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
TESTS = Path(__file__).resolve().parent
for p in (str(ROOT), str(TESTS)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = TESTS / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsgx.so")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build(ref=True)
    return pyoracle


@pytest.fixture(scope="session")
def sgx():
    import singularity_gb300 as S
    from singularity_gb300 import build
    build.build_library()
    return S


@pytest.fixture(scope="session")
def renderer(sgx):
    r = sgx.Renderer()
    yield r
    r.close()


def uniforms_from_bytes(b) -> "object":
    from singularity_gb300 import _native as N
    return N.Uniforms.from_buffer_copy(np.asarray(b, dtype=np.uint8).tobytes())


@pytest.fixture(scope="session")
def host_vectors():
    z = np.load(GOLDEN / "reference_host_vectors.npz")
    names = json.loads(str(z["names"]))
    return z, names


@pytest.fixture(scope="session")
def cuda_goldens():
    return np.load(GOLDEN / "reference_cuda_goldens.npz")
