import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device and the built libnerfgb.so")


@pytest.fixture(scope="session")
def ng():
    """The package under test (its directory name is not an identifier)."""
    return importlib.import_module("nerf-tf2_gb300")


@pytest.fixture(scope="session")
def oracle():
    return importlib.import_module("oracle")


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu-marked test needs a CUDA device")
    return torch.device("cuda", 0)
