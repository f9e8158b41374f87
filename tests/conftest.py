import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on the CPU")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def ref():
    from oracle.oracle import RefLib
    try:
        return RefLib()
    except FileNotFoundError:
        pytest.skip("the reference's host build (oracle/_ref) is not available")


@pytest.fixture(scope="session")
def lib():
    from bubbledynamics_gb300 import api
    return api.load()


@pytest.fixture(scope="session")
def ctx():
    import torch  # noqa: F401  (CUDA availability check only)
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from bubbledynamics_gb300 import api
    c = api.Context(0)
    yield c
    c.close()


def golden_path(name):
    return os.path.join(ROOT, "tests", "golden", name)
