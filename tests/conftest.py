import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "drop-of-blood_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libdropfluid.so")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def gpu_lib():
    from dropfluid import build, load
    build.build()
    return load()
