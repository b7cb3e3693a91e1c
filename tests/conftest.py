"""pytest configuration: the ``gpu`` marker (tests that need a CUDA device run only with
``-m gpu``), a per-test seeded ``rng`` (seeded from the test node id, so every test reproduces
alone), and the library built in-tree before GPU tests."""
from __future__ import annotations

import os
import sys
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device and the sm_103a library")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture
def rng(request):
    return np.random.default_rng(zlib.crc32(request.node.nodeid.encode()))


@pytest.fixture(scope="session")
def cuda_lib():
    """The built library on a CUDA device; GPU tests fail (not skip) if it is missing."""
    import torch
    from conatus_gb300 import build
    build.build()
    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    from conatus_gb300 import _lib
    return _lib.lib()


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)
