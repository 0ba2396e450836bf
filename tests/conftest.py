import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def built_library():
    """Builds (if stale) and returns the path of the CUDA library."""
    from helio_gb300 import build

    return build.build()


@pytest.fixture(scope="session")
def ctx(built_library):
    """A library context on cuda:0. GPU tests fail loudly when it cannot be made."""
    import torch

    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    from helio_gb300 import native as N

    c = N.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.build()
    return oracle
