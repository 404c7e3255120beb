import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.lib()
    return O


@pytest.fixture(scope="session")
def gpu():
    """The GPU library; the test fails (no fallback) when it cannot run."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("a gpu-marked test ran without a CUDA device")
    from buff_gb300 import capi

    capi.lib()
    torch.cuda.init()
    return capi


@pytest.fixture(scope="session")
def readme_input():
    """Path of the reference's README input (randomwalkdatasample1k-1k),
    decompressed from the committed copy under tests/golden/."""
    from tests.golden.make_golden import fixture_path

    return fixture_path()
