import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the oracle (test infrastructure) once per session; the CUDA
    library is built by __graft_entry__.build() or on demand here."""
    from oracle import oracle
    oracle.build()
    import rootpwa_gb300.build as b
    if not os.path.exists(b.LIB):
        b.build()
    yield
