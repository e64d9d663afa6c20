import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def tg():
    return importlib.import_module("tinker-gpu_gb300")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load the CUDA library; GPU tests only."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without CUDA")
    b = importlib.import_module("tinker-gpu_gb300.build")
    b.build()
    abi = importlib.import_module("tinker-gpu_gb300.abi")
    abi.load()
    return abi
