import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


@pytest.fixture(scope="session")
def native():
    """Builds (if needed) and loads libresvg_gb300.so."""
    from resvg_gb300 import build as B
    B.build()
    import resvg_gb300
    return resvg_gb300


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def gpu(native):
    try:
        import torch
        if not torch.cuda.is_available():
            pytest.skip("no CUDA device")
    except ImportError:
        pass
    native.init(0)
    return native
