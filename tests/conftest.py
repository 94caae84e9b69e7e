"""Shared test setup: the `gpu` marker, import paths and the device fixture.

Tests marked `gpu` run on a GB300 and call the native library through its C
ABI; everything else runs on the CPU (oracle, host logic, library loading).
"""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


@pytest.fixture(scope="session")
def native_lib():
    """The built libmpla.so (built on demand; no GPU needed to load it)."""
    import mpla_gb300
    from mpla_gb300 import _build

    if not mpla_gb300.LIB_PATH.exists():
        _build.build()
    return mpla_gb300.lib()


@pytest.fixture(scope="session")
def gpu(native_lib):
    """Initialised device 0; fails loudly when no GPU is present."""
    import mpla_gb300

    mpla_gb300.init(0)
    return mpla_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.lib()
    return oracle


@pytest.fixture(params=[0, 1], ids=["tensor", "simt"])
def mixed_kind(gpu, request):
    """Run a mixed-precision test with each matvec kernel (MIXED_TENSOR,
    MIXED_SIMT), restoring the library-wide choice afterwards."""
    old = gpu.get_mixed_matvec()
    gpu.set_mixed_matvec(request.param)
    yield request.param
    gpu.set_mixed_matvec(old)
