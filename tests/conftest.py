import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libsteps_gb300.so")


@pytest.fixture(scope="session")
def port():
    import pyoracle
    return pyoracle.Port()


@pytest.fixture(scope="session")
def engine():
    import steps_gb300 as S
    eng = S.Engine(0)
    yield eng
