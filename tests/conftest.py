import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the library's kernels)")


@pytest.fixture(scope="session", autouse=True)
def _built_library():
    """Build libgfpdb.so (and the C oracle) once per session if missing."""
    from flexpushdowndb_gb300._abi import LIB_PATH

    if not LIB_PATH.exists() or os.environ.get("GFPDB_REBUILD"):
        import __graft_entry__

        __graft_entry__.build()
    yield


@pytest.fixture(scope="session")
def gpu():
    """Initialise device 0 for GPU tests; a GPU test without a device fails."""
    from flexpushdowndb_gb300 import ops

    ops.init(0)
    return 0
