"""Test configuration: import paths and the `gpu` marker.

Tests marked `gpu` need a CUDA device and call the library through its C ABI;
everything else runs on the CPU (oracle, golden vectors, host logic, symbol
exports).
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT / "bb-temp-testing_gb300", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def vm():
    import voromesh_gb300

    voromesh_gb300.load()
    return voromesh_gb300
