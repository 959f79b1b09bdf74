import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "aerial-3d-model_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


_RECORD = {}


@pytest.fixture(scope="session")
def parity_record():
    """Measured deviations the parity tests report (name -> dict).  Written
    as JSON to $BA_PARITY_RECORD (a file path) at the end of the session when
    that variable is set, and printed in the terminal summary."""
    return _RECORD


def pytest_terminal_summary(terminalreporter):
    if not _RECORD:
        return
    terminalreporter.write_sep("-", "measured parity deviations")
    for k, v in sorted(_RECORD.items()):
        terminalreporter.write_line(f"{k}: {json.dumps(v)}")
    path = os.environ.get("BA_PARITY_RECORD")
    if path:
        with open(path, "w") as f:
            json.dump(_RECORD, f, indent=1, sort_keys=True)
