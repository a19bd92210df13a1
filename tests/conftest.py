import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the oracle (and the engine, which CPU tests load for its host-only
    entry points) once per session if they are missing or stale."""
    from code_mojo_gb300 import build
    build.build_oracle()
    if os.environ.get("BFGPU_SKIP_ENGINE_BUILD") != "1":
        build.build_engine()
    yield


def gpu_available() -> bool:
    try:
        import torch  # noqa: F401
        return bool(torch.cuda.is_available())
    except Exception:
        return False
