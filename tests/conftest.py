import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the module's kernels")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def module():
    """The GPU module, initialised once per session on cuda:0."""
    import simstack_gb300 as sg

    return sg.Module(0, 2 << 30)
