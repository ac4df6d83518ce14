import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the compiled engine library")


@pytest.fixture(scope="session")
def engine_lib():
    """The compiled engine; GPU tests fail (not skip) when it cannot be built or loaded."""
    import fideslib_gb300 as F
    from fideslib_gb300 import build as B
    B.build()
    return F.lib()
