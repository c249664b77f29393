import json
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the library and the oracle port once per session (no GPU needed)."""
    from qtorch_gb300 import build as qbuild
    qbuild.build()
    from oracle import port
    port.build()
    yield


@pytest.fixture(scope="session")
def ctx():
    import gc

    import qtorch_gb300 as qg
    c = qg.Context(0)
    yield c
    gc.collect()   # networks and plans release their device tensors before the context goes
    c.synchronize()
    c.close()
