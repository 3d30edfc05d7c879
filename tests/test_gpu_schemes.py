"""The pxt16, gass18 and dtred method wrappers on the GPU against the CPU
oracle: FP64 handles bit for bit (tendencies and RK4 runs, alone and with
APVM and diffusion); FP32 handles (the generic variant-0 kernels with the
branches' coefficients folded in FP64, and the cell-centred variants:
pered's coefficients and gass18's connecting edges by cell, dtred's Perot
vectors by triangle) within FP32 round-off of the oracle; the options such handles or a mesh without ed_nr cannot take are
refused."""
import ctypes

import numpy as np
import pytest

import oracle
from imodel_gb300 import _capi, fields, swm
from imodel_gb300.swm import SWM, SWMError

pytestmark = pytest.mark.gpu

SCHEMES = ("pxt16", "gass18", "dtred")
# FP32 against the FP64 oracle, relative: the tendency (max / max) and a
# 1.7-day run (L2).  Measured on a GB300: tendencies 9e-7 (mass) and
# 3e-6 to 5e-6 (momentum), runs h 4e-8, u 6e-7 to 8e-7; bounds about 5-10x
FP32_TEND = 2e-5
FP32_RUN_H, FP32_RUN_U = 4e-7, 8e-6


@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("level", [2, 4, 5])
def test_tendency_bitwise(grid_at, scheme, level):
    g = grid_at(level)
    h, u = swm.initialize_fields_tc2(g)
    rng = np.random.default_rng(level)
    h = h + rng.normal(0, 5.0, g.nv)   # unbalanced: all terms active
    u = u + rng.normal(0, 2.0, g.ne)
    m = SWM(g, "fp64", scheme=scheme)
    mg, ug = m.tendency(h, u)
    mr, ur = oracle.Oracle(g, 2, scheme=scheme).tendency(h, u)
    assert np.array_equal(mg, mr), np.max(np.abs(mg - mr))
    assert np.array_equal(ug, ur), np.max(np.abs(ug - ur))
    m.close()


@pytest.mark.parametrize("scheme", SCHEMES)
def test_balanced_state_run_bitwise(grid_at, scheme):
    """160 RK4 steps (1.7 days) of a seeded balanced state at level 4."""
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=16, seed=21)
    m = SWM(g, "fp64", scheme=scheme)
    m.set_state(h, u)
    m.advance(900.0, 160)
    hg, ug = m.get_state()
    d = m.diagnostics()
    m.close()
    o = oracle.Oracle(g, 2, scheme=scheme)
    hr, ur = o.run(h, u, 900.0, 160)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur), (
        np.max(np.abs(hg - hr)), np.max(np.abs(ug - ur)))
    o.tendency(hr, ur)
    # the diagnostics come from the last stage input in both
    mass0 = float(np.sum(g.hx_areag * h) / np.sum(g.hx_areag))
    assert abs(d["mass"] - mass0) <= 1e-13 * mass0


@pytest.mark.parametrize("scheme", SCHEMES)
def test_with_apvm_and_diffusion_bitwise(grid_at, scheme):
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=22)
    dt = 600.0
    m = SWM(g, "fp64", scheme=scheme)
    m.set_apvm(0.5, dt)
    m.set_diffusion(1.0e5, 1.0e13)
    o = oracle.Oracle(g, 2, scheme=scheme, pvspar=0.5, dt=dt, k2=1.0e5, k4=1.0e13)
    hg, ug = m.ode_rk4(h, u, dt, 6)
    hr, ur = o.run(h, u, dt, 6)
    assert np.array_equal(hg, hr) and np.array_equal(ug, ur)
    m.close()


def test_launch_counts(grid_at):
    g = grid_at(3)
    base = SWM(g, "fp64").launch_count(1)
    assert SWM(g, "fp64", scheme="pxt16").launch_count(1) == base
    assert SWM(g, "fp64", scheme="gass18").launch_count(1) == base
    assert SWM(g, "fp64", scheme="dtred").launch_count(1) == base + 4


def rel_max(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def rel_l2(a, b, w):
    return float(np.sqrt(np.sum(w * (a - b) ** 2) / np.sum(w * b * b)))


# (scheme, FP32 variant): every wrapper runs in all three
FP32_CASES = [(s, v) for s in SCHEMES for v in (0, 1, 2)]


@pytest.mark.parametrize("scheme,variant", FP32_CASES)
@pytest.mark.parametrize("level", [3, 5])
def test_fp32_tendency_against_the_oracle(grid_at, scheme, variant, level):
    """Every term of the FP32 branch (depth at the triangles, q_e, the
    kinetic energy, the PV flux) against the FP64 oracle on an unbalanced
    state."""
    g = grid_at(level)
    h, u = swm.initialize_fields_tc2(g)
    rng = np.random.default_rng(level + 10)
    h = h + rng.normal(0, 5.0, g.nv)
    u = u + rng.normal(0, 2.0, g.ne)
    m = SWM(g, "fp32", scheme=scheme)
    m.set_tuning(variant=variant)
    mg, ug = m.tendency(h, u)
    m.close()
    mr, ur = oracle.Oracle(g, 2, scheme=scheme).tendency(h, u)
    em, eu = rel_max(mg, mr), rel_max(ug, ur)
    print(f"{scheme} variant {variant} level {level}: FP32 tendency vs oracle (max / max) "
          f"mass {em:.1e}, momentum {eu:.1e}")
    assert em < FP32_TEND and eu < FP32_TEND


@pytest.mark.parametrize("scheme,variant", FP32_CASES)
def test_fp32_run_against_the_oracle(grid_at, scheme, variant):
    """320 RK4 steps (1.7 days) of a seeded balanced state at level 5."""
    g = grid_at(5)
    h, u = fields.balanced_state(g, lmax=24, seed=23)
    m = SWM(g, "fp32", scheme=scheme)
    m.set_tuning(variant=variant)
    # four kernels per stage in variant 0; the cell-centred three, plus the
    # edge pre-pass of gass18's rhombus PV (pxt16's q_e is formed in its
    # cell kernel, dtred's PV flux by its triangles)
    assert m.launch_count(1) == (16 if variant == 0 or scheme == "gass18" else 12)
    m.set_state(h, u)
    m.advance(450.0, 320)
    hg, ug = m.get_state()
    m.close()
    hr, ur = oracle.Oracle(g, 2, scheme=scheme).run(h, u, 450.0, 320)
    eh, eu = rel_l2(hg, hr, g.hx_areag), rel_l2(ug, ur, g.ed_leng * g.edhx_leng)
    dh = rel_l2(hr, h, g.hx_areag)
    print(f"{scheme} variant {variant}: FP32 vs FP64 oracle after 320 steps h {eh:.1e}, "
          f"u {eu:.1e} (the flow itself changed h by {dh:.1e})")
    assert eh < FP32_RUN_H and eu < FP32_RUN_U


@pytest.mark.parametrize("variant", [0, 1])
def test_fp32_with_apvm(grid_at, variant):
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=24)
    dt = 600.0
    m = SWM(g, "fp32", scheme="pxt16")
    m.set_apvm(0.5, dt)
    m.set_tuning(variant=variant)
    hg, ug = m.ode_rk4(h, u, dt, 48)
    m.close()
    hr, ur = oracle.Oracle(g, 2, scheme="pxt16", pvspar=0.5, dt=dt).run(h, u, dt, 48)
    eh, eu = rel_l2(hg, hr, g.hx_areag), rel_l2(ug, ur, g.ed_leng * g.edhx_leng)
    print(f"pxt16 + apvm, variant {variant}: FP32 vs FP64 oracle after 48 steps h {eh:.1e}, "
          f"u {eu:.1e}")
    assert eh < FP32_RUN_H and eu < FP32_RUN_U


@pytest.mark.parametrize("scheme", SCHEMES)
@pytest.mark.parametrize("variant", [1, 2])
def test_fp32_cell_centred_with_apvm_and_diffusion(grid_at, scheme, variant):
    """Each wrapper in the cell-centred variants with APVM, Laplacian and
    hyperdiffusion on, against the FP64 oracle of the same options."""
    g = grid_at(4)
    h, u = fields.balanced_state(g, lmax=12, seed=25)
    dt = 600.0
    m = SWM(g, "fp32", scheme=scheme)
    m.set_apvm(0.5, dt)
    m.set_diffusion(1.0e5, 1.0e13)
    m.set_tuning(variant=variant)
    hg, ug = m.ode_rk4(h, u, dt, 24)
    m.close()
    hr, ur = oracle.Oracle(g, 2, scheme=scheme, pvspar=0.5, dt=dt, k2=1.0e5,
                           k4=1.0e13).run(h, u, dt, 24)
    eh, eu = rel_l2(hg, hr, g.hx_areag), rel_l2(ug, ur, g.ed_leng * g.edhx_leng)
    print(f"{scheme} + apvm + diffusion, variant {variant}: FP32 vs FP64 oracle after 24 steps "
          f"h {eh:.1e}, u {eu:.1e}")
    assert eh < FP32_RUN_H and eu < FP32_RUN_U


def test_refusals(grid_at):
    g = grid_at(3)
    # every wrapper runs in every FP32 variant; the learned corrections are
    # built on trsk10
    for scheme in SCHEMES:
        m = SWM(g, "fp32", scheme=scheme)
        for v in (1, 2, 0):
            m.set_tuning(variant=v)
        m.close()
    with pytest.raises(SWMError) as e:
        SWM(g, "fp32", scheme="gass18", learned_params=np.zeros(100, dtype=np.float32))
    assert e.value.code == _capi.EINVAL
    # a mesh without ed_nr cannot feed pered / dtred / the circumcentres
    mesh = _capi.Mesh.from_buffer_copy(g.c_struct())  # the grid's own struct stays intact
    mesh.ed_nr = None
    opts = _capi.Opts()
    opts.precision = _capi.FP64
    opts.testcase = 2
    opts.scheme = _capi.SCHEMES["gass18"]
    h = ctypes.c_void_p()
    lib = _capi.swm_lib()
    rc = lib.imodel_swm_create(ctypes.byref(mesh), ctypes.byref(opts),
                               ctypes.byref(h))
    assert rc == _capi.EINVAL
    lib.imodel_swm_destroy(h)
    opts.scheme = 9
    rc = lib.imodel_swm_create(ctypes.byref(g.c_struct()), ctypes.byref(opts),
                               ctypes.byref(h))
    assert rc == _capi.EINVAL
    lib.imodel_swm_destroy(h)


def test_gass_divide_guard(grid_at):
    """An all-zero depth trips scalar_elem_divide's guard (swm_operators.f90:
    1604-1606) in the triangle PV and the rhombus PV alike."""
    g = grid_at(2)
    m = SWM(g, "fp64", scheme="gass18")
    with pytest.raises(SWMError) as e:
        m.tendency(np.zeros(g.nv), np.zeros(g.ne))
    assert e.value.code == _capi.EDIVZERO
