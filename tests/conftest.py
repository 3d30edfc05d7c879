"""Shared fixtures: built libraries and cached grids."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Builds the grid builder, the oracle and (where nvcc exists) the CUDA
    library once per session."""
    from imodel_gb300 import _build
    import oracle
    _build.build_mesh_lib()
    oracle.build()
    try:
        _build.build_swm_lib()
    except RuntimeError as exc:  # no nvcc: only CPU tests can run
        if "nvcc not found" not in str(exc):
            raise
    yield


_GRIDS = {}


@pytest.fixture(scope="session")
def grid_at():
    from imodel_gb300.mesh import meshbuild

    def get(level, pos="eqs"):
        key = (level, pos)
        if key not in _GRIDS:
            _GRIDS[key] = meshbuild(level, pos)
        return _GRIDS[key]
    return get


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
