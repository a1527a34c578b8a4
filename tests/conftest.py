import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine's kernels)")


@pytest.fixture(scope="session")
def engine_lib():
    from xyce_gb300 import build, engine
    if not os.path.exists(engine.LIB_PATH):
        build.build_engine()
    return engine.lib()


@pytest.fixture(scope="session")
def oracle_lib():
    from xyce_gb300 import build
    build.build_oracle()
    from oracle import oracle
    return oracle.lib()


@pytest.fixture(scope="session")
def gpu_ctx(engine_lib):
    from xyce_gb300 import engine
    return engine.Context(0)
