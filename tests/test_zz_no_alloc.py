"""The allocation-free weighted sums against the allocating diagnostics.

imodel_swm_weighted_sums_noalloc serves callers that cannot call cudaMalloc
(a host whose device memory belongs to another runtime's pool, a plugin
restricted to its caller's buffers): its block
partials live in a fixed array built into the library.  Here it is called
through the C ABI on device arrays and must agree with what
imodel_swm_diagnostics and imodel_swm_errors (which reduce into a buffer
their handle allocated) report for the same state, on two calls in a row.
The test itself allocates its device arrays with the CUDA runtime; only the
entry point under test must not.  This file is collected last so that a
failure here comes after every other test has run.
"""
import ctypes
import os

import numpy as np
import pytest

from imodel_gb300 import _build, _capi, swm
from imodel_gb300.swm import SWM

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # as tests/test_gpu_parity.py::test_diagnostics_match_oracle
H2D, D2H = 1, 2


def _cudart():
    path = os.path.join(_build._cuda_lib_dir(), "libcudart.so")
    rt = ctypes.CDLL(path if os.path.exists(path) else "libcudart.so")
    rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
    rt.cudaFree.argtypes = [ctypes.c_void_p]
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    rt.cudaMemset.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t]
    rt.cudaDeviceSynchronize.argtypes = []
    return rt


def _device_copy(rt, a):
    p = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(p), a.nbytes) == 0
    assert rt.cudaMemcpy(p, a.ctypes.data, a.nbytes, H2D) == 0
    return p


def test_noalloc_sums_match_diagnostics(grid_at):
    g = grid_at(7)
    h, u = swm.initialize_fields_tc2(g)
    h = h + np.random.default_rng(11).normal(0.0, 3.0, g.nv)
    m = SWM(g, "fp64")
    m.set_state(h, u)
    d = m.diagnostics()
    e = m.errors(np.zeros(g.nv), np.zeros(g.ne))  # ref = 0: L2 = sqrt(sum A h^2 / sum A)
    m.close()

    lib = _capi.swm_lib()
    rt = _cudart()
    w = _device_copy(rt, np.ascontiguousarray(g.hx_areag, dtype=np.float64))
    f = _device_copy(rt, np.ascontiguousarray(h, dtype=np.float64))
    out = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(out), 32) == 0
    host = np.empty(4)
    try:
        for call in range(2):
            assert rt.cudaMemset(out, 0xFF, 32) == 0  # NaN pattern: the call must write out
            rc = lib.imodel_swm_weighted_sums_noalloc(w, f, g.nv, out, None)
            assert rc == 0, (call, rc)
            assert rt.cudaDeviceSynchronize() == 0
            assert rt.cudaMemcpy(host.ctypes.data, out, 32, D2H) == 0
            sw, swf, swf2, fmax = host.tolist()
            assert abs(sw - 4 * np.pi) < 1e-12
            mass = swf / sw
            pe = 0.5 * g.grav * swf2            # flat bottom: PE = g/2 sum A h^2
            l2 = np.sqrt(swf2 / sw)
            assert abs(mass - d["mass"]) <= RTOL * abs(d["mass"]), (call, mass, d["mass"])
            assert abs(pe - d["penergy"]) <= RTOL * abs(d["penergy"]), (call, pe, d["penergy"])
            assert abs(l2 - e["error2_h"]) <= RTOL * e["error2_h"], (call, l2, e["error2_h"])
            assert fmax == e["errormax_h"], (call, fmax, e["errormax_h"])
    finally:
        for p in (w, f, out):
            rt.cudaFree(p)


def test_noalloc_max_keeps_nan(grid_at):
    """A NaN in the field makes the maximum NaN too (not a finite value)."""
    g = grid_at(4)
    lib = _capi.swm_lib()
    rt = _cudart()
    f_host = np.linspace(-2.0, 3.0, g.nv)
    f_host[g.nv // 3] = np.nan
    w = _device_copy(rt, np.ascontiguousarray(g.hx_areag, dtype=np.float64))
    f = _device_copy(rt, f_host)
    out = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(out), 32) == 0
    host = np.zeros(4)
    try:
        assert lib.imodel_swm_weighted_sums_noalloc(w, f, g.nv, out, None) == 0
        assert rt.cudaDeviceSynchronize() == 0
        assert rt.cudaMemcpy(host.ctypes.data, out, 32, D2H) == 0
        assert abs(host[0] - 4 * np.pi) < 1e-12
        assert np.isnan(host[1]) and np.isnan(host[3])
    finally:
        for p in (w, f, out):
            rt.cudaFree(p)


def test_noalloc_rejects_oversize_input():
    lib = _capi.swm_lib()
    too_many = 4096 * 256 * 32 + 1
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.imodel_swm_weighted_sums_noalloc(dummy, dummy, too_many, dummy, None)
    assert rc == _capi.ETOOBIG
