import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build_restatement()
    return oracle


@pytest.fixture(scope="session")
def gpu():
    """The GPU library, built in-tree; a GPU test fails loudly if it cannot load."""
    import imfit_gb300
    from imfit_gb300 import build
    build.build()
    imfit_gb300.load_library()
    return imfit_gb300


GOLDEN = os.path.join(ROOT, "tests", "golden")
