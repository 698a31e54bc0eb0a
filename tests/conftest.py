import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the CUDA path)")
    config.addinivalue_line("markers", "slow: long CPU oracle run, enabled with PFC_SLOW=1")


def pytest_collection_modifyitems(config, items):
    if os.environ.get("PFC_SLOW") == "1":
        return
    skip = pytest.mark.skip(reason="slow oracle case; set PFC_SLOW=1 to run")
    for it in items:
        if "slow" in it.keywords:
            it.add_marker(skip)
