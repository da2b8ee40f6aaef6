"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on
the CPU (oracle, host logic, ABI exports)."""
import os
import pathlib
import sys

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The native library on cuda:0 (built for sm_103a).  No fallback."""
    import cappgpu
    cappgpu.build()
    lib = cappgpu.Library()
    yield lib
    lib.finalize()
