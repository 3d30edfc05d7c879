"""A compiled host program on the C ABI (tests/c/swm_driver.c: the grid,
a handle and the swm_tests time loop, one imodel_swm_step per RK4 step on
host arrays), standing in for the reference's Fortran driver: it compiles
and links against the in-tree libraries with the headers alone (CPU), and
on the GPU its FP64 run equals the Python path and the oracle bit for bit
and its FP32 run stays within FP32 round-off."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from imodel_gb300 import _capi, swm

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "swm_driver.c")
LIB = os.path.join(ROOT, "imodel_gb300", "_lib")


def _build(tmp_path):
    for name in ("libimodel_swm.so", "libimodel_mesh.so"):
        if not os.path.exists(os.path.join(LIB, name)):
            pytest.skip(f"{name} is not built")
    exe = str(tmp_path / "swm_driver")
    subprocess.run(["gcc", "-std=c11", "-O2", "-I", os.path.join(ROOT, "include"), SRC,
                    "-L", LIB, "-limodel_swm", "-limodel_mesh", "-Wl,-rpath," + LIB, "-o", exe],
                   check=True, capture_output=True, text=True)
    return exe


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a C compiler")
def test_driver_compiles_and_links(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_driver_time_loop(tmp_path, grid_at, precision):
    import oracle
    exe = _build(tmp_path)
    level, dt, n = 4, 600.0, 24
    g = grid_at(level)
    h, u = swm.initialize_fields_tc2(g)
    hin, uin = tmp_path / "h0.bin", tmp_path / "u0.bin"
    hout, uout = tmp_path / "h1.bin", tmp_path / "u1.bin"
    h.astype(np.float64).tofile(hin)
    u.astype(np.float64).tofile(uin)
    prec = {"fp64": _capi.FP64, "fp32": _capi.FP32}[precision]
    r = subprocess.run([exe, str(level), str(prec), str(n), str(dt), "8", str(hin), str(uin),
                        str(hout), str(uout), "0"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert len(r.stdout.splitlines()) == n // 8
    hc, uc = np.fromfile(hout), np.fromfile(uout)
    hr, ur = oracle.Oracle(g, 2).run(h, u, dt, n)
    if precision == "fp64":
        hp, up = swm.SWM(g, "fp64").ode_rk4(h, u, dt, n)
        assert np.array_equal(hc, hp) and np.array_equal(uc, up)
        assert np.array_equal(hc, hr) and np.array_equal(uc, ur)
    else:
        eh = np.sqrt(np.sum(g.hx_areag * (hc - hr) ** 2) / np.sum(g.hx_areag * hr ** 2))
        assert eh < 1e-6, eh
