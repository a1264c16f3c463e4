import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
TESTS = Path(__file__).resolve().parent
if str(TESTS) not in sys.path:
    sys.path.insert(0, str(TESTS))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session")
def golden():
    return json.loads((ROOT / "tests" / "golden" / "reference_cases.json").read_text())


@pytest.fixture(scope="session")
def rl():
    """The product library; built in-tree if it is missing (nvcc cross-compiles here)."""
    import __graft_entry__
    __graft_entry__._build_module().build_library()
    import rulinalg_gb300
    return rulinalg_gb300


@pytest.fixture(scope="session")
def gpu(rl):
    if not rl.device_available():
        pytest.fail("no usable sm_103 GPU: the GPU tests need one (there is no CPU fallback)")
    return rl
