import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
    """Build (if stale) and load libhydrant_gb300.so."""
    from hydrant_gb300 import build as hb

    hb.build()
    import hydrant_gb300 as hy

    return hy.lib()


@pytest.fixture(scope="session")
def ctx(built_lib):
    import hydrant_gb300 as hy

    c = hy.Context(0)
    yield c
    c.close()
