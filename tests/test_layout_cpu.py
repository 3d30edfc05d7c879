"""The device layout the step handles build (host code, no GPU use): every
array is the same whatever the number of host threads, for each method
wrapper, and a broken mesh is refused the same way."""
import ctypes

import numpy as np
import pytest

from imodel_gb300 import _capi


def _digest(mesh, scheme, nthreads):
    h = ctypes.c_uint64()
    rc = _capi.swm_lib().imodel_swm_test_layout_digest(ctypes.byref(mesh), scheme, nthreads,
                                                        ctypes.byref(h))
    return rc, h.value


@pytest.mark.parametrize("scheme", [0, 1, 2, 3])
def test_layout_does_not_depend_on_the_thread_count(grid_at, scheme):
    g = grid_at(5)
    mesh = g.c_struct()
    got = [_digest(mesh, scheme, n) for n in (1, 3, 0)]
    assert all(rc == 0 for rc, _ in got)
    assert got[0][1] == got[1][1] == got[2][1]


def test_broken_mesh_is_refused_with_any_thread_count(grid_at):
    g = grid_at(3)
    mesh = _capi.Mesh.from_buffer_copy(g.c_struct())  # the grid's own struct stays intact
    v_ed = np.array(g.v_ed, dtype=np.int32)
    v_ed[17, 2] = 0                                    # an edge index out of range
    mesh.v_ed = _capi.as_i32p(v_ed)
    for n in (1, 0):
        assert _digest(mesh, 0, n)[0] == _capi.EINVAL
