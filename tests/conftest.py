import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "nemo-fmi-devel_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def gyre1():
    from nemo_gpu import gyre
    dom = gyre.domain(1)
    nam = gyre.namelist()
    return dom, nam


def pytest_sessionfinish(session, exitstatus):
    """Write the pointwise parity statistics (tests/harness.py REPORT) to the JSON
    file named by $NEMO_PARITY_REPORT, when that is set."""
    path = os.environ.get("NEMO_PARITY_REPORT")
    if not path:
        return
    try:
        import json

        from harness import REPORT
    except Exception:
        return
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "w") as f:
        json.dump(REPORT, f, indent=1, sort_keys=True)
