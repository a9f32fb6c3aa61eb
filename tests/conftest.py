"""Shared fixtures: the native library, the CPU oracle, the gpu marker."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and runs the native kernels")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def native():
    from voidray_gb300 import build as vb

    vb.build()
    import voidray_gb300 as vr

    return vr


@pytest.fixture(scope="session")
def gpu(native):
    if not native.lib().vr_device_available():
        pytest.fail("GPU test without a usable CUDA device")
    return native
