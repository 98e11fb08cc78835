"""Shared test set-up: markers, import paths, built libraries, cases."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("bte-barna_gb300", "oracle"):
    p = os.path.join(REPO, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300)")


@pytest.fixture(scope="session")
def built():
    """Build the engine (sm_103a cross-compile works without a GPU) and the oracle."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "bte_engine_build", os.path.join(REPO, "bte-barna_gb300", "build.py"))
    engine_build = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(engine_build)
    lib = engine_build.build()
    import pyoracle
    pyoracle.load()
    return lib


@pytest.fixture(scope="session")
def engine(built):
    import btegpu
    e = btegpu.Engine(0)
    yield e
    e.close()
