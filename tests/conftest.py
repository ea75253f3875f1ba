import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ac-dc_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for p in (ROOT, PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    import build as acdc_build  # ac-dc_gb300/build.py
    import oracle
    acdc_build.build_all()
    oracle.build()


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    _ensure_built()
    yield


@pytest.fixture(scope="session")
def ctx():
    import acdc
    c = acdc.Context(0)
    yield c
    import gc
    gc.collect()  # problems hold the context; destroy it after they are gone
    c.close()
