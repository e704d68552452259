import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libdrawgpu.so")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    from oracle import build as ob

    ob.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_ctx():
    from draw_gb300 import _build

    _build.build()
    from draw_gb300 import renderer

    ctx = renderer.Context(0)
    yield ctx
    ctx.close()
