"""The C-ABI libraries load and export every symbol the headers declare.
No compute call is made: these run without a GPU."""
import ctypes
import os
import re

import pytest

from imodel_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    with open(os.path.join(ROOT, "include", header)) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(imodel_\w+)\s*\(", text)))


def test_header_lists_match_python_mirror():
    assert _declared("imodel_mesh.h") == sorted(_capi.MESH_SYMBOLS)
    assert _declared("imodel_swm.h") == sorted(_capi.SWM_SYMBOLS)


def test_mlp_header_matches_python_mirror():
    assert _declared("imodel_mlp.h") == sorted(_capi.MLP_SYMBOLS)
    assert _declared("imodel_moist.h") == sorted(_capi.MOIST_SYMBOLS)


def test_mesh_library_exports():
    lib = _capi.mesh_lib()
    for name in _declared("imodel_mesh.h"):
        assert hasattr(lib, name), name


def test_swm_library_exports():
    path = _capi.lib_path("libimodel_swm.so")
    if not os.path.exists(path):
        pytest.skip("CUDA library not built (no nvcc)")
    lib = ctypes.CDLL(path)
    for name in _declared("imodel_swm.h") + _declared("imodel_mlp.h") + \
            _declared("imodel_moist.h"):
        assert hasattr(lib, name), name


def test_struct_sizes_match_c():
    # 3 int32 + 25 pointers (padded to 8) + 3 doubles
    assert ctypes.sizeof(_capi.Mesh) == 16 + 25 * 8 + 24
    assert ctypes.sizeof(_capi.Diag) == 8 * 8 + 8


def test_null_arguments_are_rejected_without_device():
    lib = _capi.swm_lib()
    h = ctypes.c_void_p()
    assert lib.imodel_swm_create(None, None, ctypes.byref(h)) == _capi.EINVAL
    assert b"NULL" in lib.imodel_swm_last_error(h)
    lib.imodel_swm_destroy(h)
    assert lib.imodel_swm_step(None, None, None, 1.0, 1) == _capi.EINVAL
