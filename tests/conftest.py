import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    # Build the native library and the oracle once per session if missing or stale.
    from govid_gb300 import build as b

    b.build()
    import ebiv_oracle

    ebiv_oracle.build()


def has_gpu() -> bool:
    from govid_gb300 import ebiv

    return ebiv.device_available()


@pytest.fixture(scope="session")
def gpu_required():
    if not has_gpu():
        pytest.fail("no usable CUDA device: GPU tests must run on a GB300")
