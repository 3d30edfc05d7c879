"""The GPU back end of the grid builder (imodel_mesh_build_gpu).

* the grid it returns has the host builder's numbering, signs and node
  positions exactly (the numbering built by GPU kernels), and its lengths, areas, angles, kite fractions and TRSK weights within a
  few units in the last place of the host values (the GPU's atan, tan, atan2
  and asin against the host C library's; every other operation rounds the
  same way);
* the Delaunay check finds the same (no) violations;
* the FP64 step on a GPU-built grid equals the oracle on that grid bit for
  bit, and differs from the step on the host-built grid at round-off only.
"""
import time

import numpy as np
import pytest

import oracle
from imodel_gb300 import fields, mesh
from imodel_gb300.mesh import meshbuild
from imodel_gb300.swm import SWM

pytestmark = pytest.mark.gpu

INTS = list(mesh._I32) + list(mesh._EXTRA_I32)
FLOATS = list(mesh._F64) + list(mesh._EXTRA_F64)
EPS = np.finfo(np.float64).eps


def ulps_of_scale(a, b):
    """max |a - b| in units of eps times the array's largest magnitude."""
    scale = max(float(np.max(np.abs(a))), float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / (EPS * scale)


def compare(gh, gg):
    for k in INTS:
        assert np.array_equal(getattr(gh, k), getattr(gg, k)), k
    # the subdivision's midpoints round as on the host
    assert np.array_equal(gh.v_p, gg.v_p)
    worst = {}
    for k in FLOATS:
        a, b = getattr(gh, k), getattr(gg, k)
        assert a.shape == b.shape, k
        assert np.all(np.isfinite(b)), k
        worst[k] = ulps_of_scale(a, b)
    return worst


@pytest.mark.parametrize("pos", ["eqs", "pol"])
@pytest.mark.parametrize("level", [0, 1, 2, 3, 4, 5, 6, 7])
def test_gpu_geometry_equals_the_host_build(pos, level):
    gh = meshbuild(level, pos)
    gg = meshbuild(level, pos, device=0)
    worst = compare(gh, gg)
    top = sorted(worst.items(), key=lambda kv: -kv[1])[:3]
    print(f"{pos} level {level}: largest differences (eps x array scale): "
          + ", ".join(f"{k} {v:.1f}" for k, v in top))
    for k, v in worst.items():
        assert v <= 64.0, (k, v)
    assert gg.delaunay_violations == gh.delaunay_violations == 0
    assert gg.delaunay_margin == pytest.approx(gh.delaunay_margin, rel=1e-9)


def test_gpu_build_at_level_9_and_its_time():
    t0 = time.perf_counter()
    gh = meshbuild(9)
    t1 = time.perf_counter()
    gg = meshbuild(9, device=0)
    t2 = time.perf_counter()
    worst = compare(gh, gg)
    print(f"level 9: host build {t1 - t0:.2f} s, GPU build {t2 - t1:.2f} s; "
          f"largest difference {max(worst.values()):.1f} eps x scale")
    assert max(worst.values()) <= 64.0
    assert gg.delaunay_violations == 0


def test_step_on_a_gpu_built_grid():
    gg = meshbuild(5, device=0)
    gh = meshbuild(5)
    h, u = fields.balanced_state(gh, lmax=16, seed=41)
    m = SWM(gg, "fp64")
    hg, ug = m.ode_rk4(h, u, 600.0, 24)
    m.close()
    hr, ur = oracle.Oracle(gg, 2).run(h, u, 600.0, 24)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)
    m = SWM(gh, "fp64")
    hh, uh = m.ode_rk4(h, u, 600.0, 24)
    m.close()
    dh = float(np.max(np.abs(hg - hh)) / np.max(np.abs(hh)))
    du = float(np.max(np.abs(ug - uh)) / np.max(np.abs(uh)))
    print(f"24 steps on the GPU-built vs the host-built level-5 grid: h {dh:.1e}, u {du:.1e}")
    assert dh < 1e-12 and du < 1e-10


def test_invalid_arguments():
    lib = mesh._capi.mesh_lib()
    import ctypes
    h = ctypes.c_void_p()
    assert lib.imodel_mesh_build_gpu(12, 0, 0, ctypes.byref(h)) == mesh._capi.EINVAL
    assert lib.imodel_mesh_build_gpu(3, 2, 0, ctypes.byref(h)) == mesh._capi.EINVAL
    assert lib.imodel_mesh_build_gpu(3, 0, -1, ctypes.byref(h)) == mesh._capi.EINVAL
    assert not h.value
