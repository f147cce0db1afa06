import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs libuww_gb300.so kernels)")


@pytest.fixture(scope="session")
def built_lib():
    """libuww_gb300.so, built in-tree if missing or stale."""
    from underwaterworld_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def oracle(built_lib):
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def ctx_factory(built_lib):
    from underwaterworld_gb300.chunk import Context
    made = []

    def make(params=None):
        c = Context(params)
        made.append(c)
        return c

    yield make
    for c in made:
        c.close()
