import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden_dir():
    return GOLDEN


def pytest_sessionfinish(session, exitstatus):
    """OSD_GB300_ERROR_REPORT=<path>: write the per-output errors the GPU parity tests saw."""
    path = os.environ.get("OSD_GB300_ERROR_REPORT")
    if not path:
        return
    import json

    import gpu_util
    with open(path, "w") as f:
        json.dump(gpu_util.REPORT, f, indent=0)
