import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = Path(__file__).resolve().parent / "golden"


def fixture_count(group: str) -> int:
    """Number of reference fixtures in a group of reference_philox.json (for
    parametrising tests at collection time)."""
    return len(json.loads((GOLDEN / "reference_philox.json").read_text())[group])


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def ref_fixtures():
    return json.loads((GOLDEN / "reference_philox.json").read_text())


@pytest.fixture(scope="session")
def example_logs():
    return json.loads((GOLDEN / "example_logs.json").read_text())
