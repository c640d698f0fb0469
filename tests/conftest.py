import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "phj-bench_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the sm_103a library)")


@pytest.fixture(scope="session")
def ctx():
    import phj_gpu

    c = phj_gpu.Context(0)
    yield c
    c.close()
