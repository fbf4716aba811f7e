"""Shared test configuration: the `gpu` marker, and the builds of the oracle and the library."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def fgl():
    from film_grain_gb300 import build
    build.build()
    import film_grain_gb300
    film_grain_gb300.lib()
    return film_grain_gb300


@pytest.fixture(scope="session")
def cuda(fgl):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    return torch
