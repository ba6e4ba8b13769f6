import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def built_lib():
    """Path of libcbx.so, building it in-tree if it is missing."""
    from cosmicblup_gb300 import build as b
    if not os.path.exists(b.LIB):
        b.build()
    return b.LIB


@pytest.fixture(scope="session")
def handle(built_lib):
    from cosmicblup_gb300 import Handle
    h = Handle(0)
    yield h
    h.close()


@pytest.fixture(scope="session")
def toy_golden():
    with open(os.path.join(GOLDEN, "toy_grm.json")) as f:
        return json.load(f)
