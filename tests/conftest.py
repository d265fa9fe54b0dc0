"""Shared test setup: the 'gpu' marker and the in-tree build."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def built_library():
    from mcac_gb300 import build
    build.build_library()
    build.build_oracle()
    return build.LIB


@pytest.fixture(scope="session")
def has_gpu():
    from mcac_gb300 import api
    return api.device_count() > 0


@pytest.fixture(autouse=True)
def _skip_gpu_without_device(request, has_gpu):
    if request.node.get_closest_marker("gpu") and not has_gpu:
        pytest.skip("no CUDA device")


def load_golden(name: str):
    return np.load(GOLDEN / name, allow_pickle=False)
