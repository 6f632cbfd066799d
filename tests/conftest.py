import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "vahana.jl_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def vh():
    """The product package with its CUDA library built (fails loudly if the
    library cannot be built or loaded)."""
    import vahana_gb300
    vahana_gb300.build()
    return vahana_gb300
