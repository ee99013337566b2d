import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Compile (or re-use) every native part once per session."""
    from blamm_gb300 import build
    build.build()
    import oracle_build  # oracle/oracle_build.py (oracle/ is on sys.path)
    oracle_build.build()
    yield


@pytest.fixture(scope="session")
def scanner():
    from blamm_gb300 import GpuScanner
    s = GpuScanner(0, "bf16x2")
    yield s
    s.close()
