import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "mesh-deform_gb300", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Compiles the CUDA library and the oracle once per session."""
    import build_lib
    from oracle import oracle

    build_lib.build()
    oracle.build()
    return True


@pytest.fixture(scope="session")
def gpu(built):
    import arap_gpu

    arap_gpu.load()
    return arap_gpu
