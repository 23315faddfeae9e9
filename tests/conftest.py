import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (str(ROOT), str(ROOT / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the engine on cuda:0)")


@pytest.fixture(scope="session")
def built():
    """Native libraries built for this machine (engine, scan generator, oracle)."""
    import __graft_entry__ as g

    g.build()
    return True
