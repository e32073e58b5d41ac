import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def ref_fixtures():
    return json.loads((GOLDEN / "reference_philox.json").read_text())


@pytest.fixture(scope="session")
def example_logs():
    return json.loads((GOLDEN / "example_logs.json").read_text())
