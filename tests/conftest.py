import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: full-size workloads (minutes of CPU oracle time)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def ctx():
    import dbd_gb300 as dbd
    c = dbd.Context(cpu_gib=64, gpu_gib=64, device=0)
    yield c
    c.close()
