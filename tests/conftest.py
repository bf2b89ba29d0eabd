"""Test configuration: the `gpu` marker and import paths.

Tests marked ``gpu`` need a CUDA device and the built library; everything else runs on
the CPU (oracle, host logic, the C ABI's exports).
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "wgpu-voxel-engine_gb300"), os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def built():
    """Builds (incrementally) the library and the oracle once per session."""
    from voxgpu import _build
    _build.build_library()
    _build.build_oracle()
    return True


@pytest.fixture(scope="session")
def oracle(built):
    import vox_oracle
    vox_oracle.load()
    return vox_oracle


@pytest.fixture(scope="session")
def vox(built):
    import voxgpu
    voxgpu.lib()
    return voxgpu
