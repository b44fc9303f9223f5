import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests"),
          os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def pgb():
    """The product package with its shared library built in-tree."""
    from pimc_gb300 import build as _build  # noqa: F401
    import pimc_gb300.build as b
    b.build()
    import pimc_gb300
    pimc_gb300._lib.load()
    return pimc_gb300
