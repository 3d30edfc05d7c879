"""State transfer between the caller's host arrays and the device.

imodel_swm_step, _set_state and _get_state read and write the caller's FP64
arrays in reference order.  Page-locked arrays (cudaMallocHost,
cudaHostRegister) are read and written by kernels over the host link, with
the permutation to device order applied on the device; pageable arrays go
through cudaMemcpyAsync and a staging buffer.  Both routes must give the
same bits, for both precisions, for arrays at an offset inside a larger
page-locked allocation, and must report a NaN written back to the host.
"""
import ctypes
import os

import numpy as np
import pytest

from imodel_gb300 import _build, _capi, swm
from imodel_gb300.swm import SWM

pytestmark = pytest.mark.gpu


def _cudart():
    path = os.path.join(_build._cuda_lib_dir(), "libcudart.so")
    rt = ctypes.CDLL(path if os.path.exists(path) else "libcudart.so")
    rt.cudaMallocHost.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
    rt.cudaFreeHost.argtypes = [ctypes.c_void_p]
    return rt


class Pinned:
    """One page-locked FP64 buffer of n values, viewed as a numpy array."""

    def __init__(self, rt, n):
        self.rt = rt
        self.p = ctypes.c_void_p()
        assert rt.cudaMallocHost(ctypes.byref(self.p), n * 8) == 0
        self.a = np.ctypeslib.as_array(ctypes.cast(self.p, ctypes.POINTER(ctypes.c_double)),
                                       shape=(n,))

    def ptr(self, offset=0):
        return ctypes.cast(self.p.value + 8 * offset, ctypes.POINTER(ctypes.c_double))

    def free(self):
        self.rt.cudaFreeHost(self.p)


@pytest.mark.parametrize("precision,level", [("fp64", 3), ("fp32", 5)])
def test_pinned_and_pageable_steps_agree(grid_at, precision, level):
    g = grid_at(level)
    h0, u0 = swm.initialize_fields_tc2(g)
    dt = 400.0 if level <= 3 else 200.0
    a = SWM(g, precision=precision)
    ha, ua = a.ode_rk4(h0, u0, dt, 3)            # pageable numpy arrays
    ha, ua = a.ode_rk4(ha, ua, dt, 1)
    b = SWM(g, precision=precision)
    rt = _cudart()
    # h and u share one page-locked allocation, u at an offset behind h
    buf = Pinned(rt, g.nv + g.ne + 3)
    try:
        buf.a[:g.nv] = h0
        buf.a[g.nv + 3:] = u0
        hp, up = buf.ptr(0), buf.ptr(g.nv + 3)
        assert b.lib.imodel_swm_step(b.handle, hp, up, dt, 3) == 0
        assert b.lib.imodel_swm_step(b.handle, hp, up, dt, 1) == 0
        assert np.array_equal(buf.a[:g.nv], ha)
        assert np.array_equal(buf.a[g.nv + 3:], ua)
        # get_state into page-locked arrays gives the same bits again
        buf.a[:] = 0.0
        assert b.lib.imodel_swm_get_state(b.handle, hp, up) == 0
        assert np.array_equal(buf.a[:g.nv], ha)
        assert np.array_equal(buf.a[g.nv + 3:], ua)
        # and set_state from them continues the same run
        assert b.lib.imodel_swm_set_state(b.handle, hp, up) == 0
        b.advance(dt, 2)
        a.set_state(ha, ua)
        a.advance(dt, 2)
        hb, ub = b.get_state()
        hc, uc = a.get_state()
        assert np.array_equal(hb, hc) and np.array_equal(ub, uc)
    finally:
        buf.free()
        a.close()
        b.close()


def test_pinned_nan_is_reported(grid_at):
    g = grid_at(3)
    h0, u0 = swm.initialize_fields_tc2(g)
    m = SWM(g, precision="fp32")
    rt = _cudart()
    hb, ub = Pinned(rt, g.nv), Pinned(rt, g.ne)
    try:
        hb.a[:] = h0
        ub.a[:] = u0
        ub.a[g.ne // 2] = np.nan
        rc = m.lib.imodel_swm_step(m.handle, hb.ptr(), ub.ptr(), 400.0, 1)
        assert rc == _capi.EBLOWUP
    finally:
        hb.free()
        ub.free()
        m.close()


def _pinned_pair(rt, h, u):
    hb, ub = Pinned(rt, h.size), Pinned(rt, u.size)
    hb.a[:] = h
    ub.a[:] = u
    return hb, ub


def test_pinned_learned_steps_match_advance(grid_at):
    """With the learned correction, imodel_swm_step on page-locked arrays runs
    the energy check beside the write-back; the states equal those of
    set_state + advance + get_state, which check after each call too."""
    from imodel_gb300 import fields, learned
    g = grid_at(5)
    h, u = fields.balanced_state(g, lmax=24, seed=5)
    p = learned.trained_params()
    assert p is not None
    a = SWM(g, "fp32", learned_params=p)
    b = SWM(g, "fp32", learned_params=p)
    rt = _cudart()
    hb, ub = _pinned_pair(rt, h, u)
    try:
        a.set_state(h, u)
        for _ in range(3):
            a.advance(450.0, 1)
            assert b.lib.imodel_swm_step(b.handle, hb.ptr(), ub.ptr(), 450.0, 1) == 0
        ha, ua = a.get_state()
        assert np.array_equal(hb.a, ha) and np.array_equal(ub.a, ua)
        assert a.diagnostics()["learned_active"] == 1
        assert b.diagnostics()["learned_active"] == 1
    finally:
        hb.free()
        ub.free()
        a.close()
        b.close()


def test_pinned_learned_trip_rolls_back(grid_at):
    """A step that breaks the drift bound inside imodel_swm_step on
    page-locked arrays is rolled back and stepped with the plain scheme."""
    from imodel_gb300 import fields
    from oracle import mlp_oracle as mo
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=16, seed=3)
    p = mo.init_params(9) * 50.0
    p[-1] = 30.0
    a = SWM(g, "fp32", learned_params=p, drift_bound=1e-12)
    b = SWM(g, "fp32")
    b.set_tuning(variant=1)
    rt = _cudart()
    hb, ub = _pinned_pair(rt, h, u)
    try:
        hc, uc = h, u
        for _ in range(3):
            assert a.lib.imodel_swm_step(a.handle, hb.ptr(), ub.ptr(), 900.0, 1) == 0
            hc, uc = b.ode_rk4(hc, uc, 900.0, 1)
        assert a.diagnostics()["learned_active"] == 0
        assert np.array_equal(hb.a, hc) and np.array_equal(ub.a, uc)
    finally:
        hb.free()
        ub.free()
        a.close()
        b.close()
