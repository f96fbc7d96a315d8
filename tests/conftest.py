import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: long-running full-size check")


@pytest.fixture(scope="session")
def sbc_lib():
    """The CUDA library, built in-tree if needed (no fallback)."""
    from streamingbc_gb300 import build, native
    if not os.path.exists(native.LIB_PATH):
        build.build()
    return native.load()


@pytest.fixture(scope="session")
def port_lib():
    from oracle import oracle as orc
    if not os.path.exists(orc.PORT_SO):
        orc.build()
    return orc
