import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")
    config.addinivalue_line("markers", "slow: longer CPU test")


@pytest.fixture(scope="session", autouse=True)
def _built(tmp_path_factory):
    """Build the native pieces once per session (fast when up to date).  The
    kernel choices persisted across processes go to a file of this session,
    so no test reads choices an earlier run left behind."""
    import os

    from fdtd_2d_gb300 import build

    os.environ["FDTD2D_TUNE_CACHE"] = str(tmp_path_factory.mktemp("tune") / "kernel_choices.json")
    build.build()
    yield


def cuda_available() -> bool:
    import fdtd_2d_gb300 as F

    return F.device_count() > 0


@pytest.fixture(scope="session")
def gpu():
    if not cuda_available():
        pytest.skip("no CUDA device")
    return 0
