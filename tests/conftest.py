import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
for sub in ("cl-ops_gb300", "oracle", "tests"):
    p = str(ROOT / sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and runs the CUDA path")
    config.addinivalue_line("markers", "slow: full-size property checks")


@pytest.fixture(scope="session")
def clops():
    import clops as m
    return m


@pytest.fixture(scope="session")
def ctx(clops):
    c = clops.Context(0)
    yield c
    c.destroy()


@pytest.fixture(scope="session")
def queue(clops, ctx):
    q = clops.Queue(ctx, profiling=True)
    yield q
    q.destroy()
