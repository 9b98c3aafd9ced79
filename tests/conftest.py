import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the oracle and the CUDA library once per session (no-ops when up to date)."""
    import importlib.util

    for path in (ROOT / "oracle" / "build.py", ROOT / "fgrain_gb300" / "build.py"):
        spec = importlib.util.spec_from_file_location(path.parent.name + "_build", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    yield


@pytest.fixture(scope="session")
def engine():
    import fgrain_gb300 as fg

    e = fg.get_gpu_engine()
    if e is None:
        pytest.fail("no usable CUDA device for a gpu-marked test")
    return e
