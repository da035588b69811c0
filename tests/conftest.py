import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT / "rivin-perm_gb300", ROOT / "oracle", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libpermgpu.so")


def golden(name):
    return json.loads((GOLDEN / name).read_text())


@pytest.fixture(scope="session")
def lib():
    """The CUDA library; GPU tests fail (never skip) when it is unusable."""
    from permgpu import _lib
    handle = _lib.load()
    assert handle.pg_cuda_runtime_available() == 1, "no usable CUDA device"
    return _lib
