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


def reference_python():
    """The reference's Python package directory (holding ``conatus/``) where it is present: the
    environment variable CONATUS_REFERENCE_PYTHON, else CONATUS_REFERENCE/python, else the tree
    that built oracle/_ref (recorded in oracle/_ref/REFERENCE by the build); None otherwise."""
    cands = [os.environ.get("CONATUS_REFERENCE_PYTHON")]
    if os.environ.get("CONATUS_REFERENCE"):
        cands.append(os.path.join(os.environ["CONATUS_REFERENCE"], "python"))
    rec = os.path.join(ROOT, "oracle", "_ref", "REFERENCE")
    if os.path.exists(rec):
        with open(rec) as f:
            cands.append(os.path.join(f.read().strip(), "python"))
    for c in cands:
        if c and os.path.exists(os.path.join(c, "conatus", "__init__.py")):
            return c
    return None
