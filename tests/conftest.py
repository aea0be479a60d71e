import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs librdn kernels)")


@pytest.fixture(scope="session", autouse=True)
def _native_libraries():
    """Builds the oracle (always) and librdn (when missing) before any test."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    from rendiation_gb300 import native

    if not os.path.exists(native.LIB_PATH):
        from rendiation_gb300 import build_native

        build_native.build()
    yield


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a CUDA device")
    return torch.device("cuda:0")
