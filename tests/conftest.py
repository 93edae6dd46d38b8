"""Test configuration: the `gpu` marker, and the checkers built on demand."""

import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the GPU path through the C ABI)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.bindings import Oracle, build_oracle

    build_oracle()
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle.bindings import REF_SO, Reference, reference_available

    if not reference_available():
        pytest.skip("reference sources not present on this host")
    try:
        return Reference()
    except Exception as e:  # pragma: no cover
        pytest.skip(f"reference library unavailable: {e}")


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library; GPU tests fail (not skip) when it is missing, so a silent fallback cannot pass."""
    from hibf_gb300 import _build, _native

    if not _native.LIB_PATH.exists():
        _build.build()
    L = _native.lib()
    if _native.device_count() == 0:
        pytest.fail("GPU test collected on a host without a CUDA device")
    return L
