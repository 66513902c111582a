import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU case")


def pytest_collection_modifyitems(config, items):
    """Cases marked ``slow`` (a CPU oracle run of minutes) run only when FF_SLOW=1."""
    if os.environ.get("FF_SLOW") == "1":
        return
    skip = pytest.mark.skip(reason="slow CPU case; set FF_SLOW=1 to run")
    for item in items:
        if "slow" in item.keywords and "gpu" not in item.keywords:
            item.add_marker(skip)
