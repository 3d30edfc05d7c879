"""Initial states of iModel's other shallow-water test cases on HTC points.

``initialize_fields`` (src/swm.f90:1134-2380) fills h, u and the bottom
topography for a test-case number.  Case 2 lives in ``swm.py``; this module
adds the cases that need nothing but closed-form fields:

* 0 -- time-discretisation check: h = cos(lon) cos^2(lat), u = 0
  (swm.f90:1135-1146);
* 1 -- solid-body rotation of a cosine bell, the advection test (momentum
  equation off; swm.f90:1148-1203);
* 5 -- zonal flow over an isolated conical mountain (Williamson et al.
  1992, case 5; swm.f90:1327-1423);
* 6 -- Rossby-Haurwitz wave of wavenumber 4 (Williamson case 6;
  swm.f90:1426-1620, height ``h_tc6`` at :2392-2413).

Every field is returned in the grid's (reference) ordering; u is the normal
component along ``ed%tg`` at the triangle-edge midpoint ``ed%c``, as the
HTC staggering of the step uses.

``tc6_exact_tendency`` gives the exact mass and momentum tendencies of the
case-6 initial state, the quantities the reference's local truncation error
harness compares the discrete operators with (``test_lterror``, case 14 of
the driver).  They are derived here from the closed-form fields: the first
derivatives of the analytic u, v and h come from complex-step
differentiation (Squire and Trapp, SIAM Review 40, 1998: f'(x) =
Im f(x + i s) / s, exact to rounding for s = 1e-30), and the tendencies from
the vector-invariant equations on the sphere.
"""
from __future__ import annotations

import numpy as np

from .mesh import DAY2SEC, ERAD, GRAV, OMEGA, PI, Grid
from .swm import convert_vec_sph2cart, dot3, initialize_fields_tc2

GRAVI = 1.0 / GRAV
PIO2 = PI / 2.0
EPS = float(np.finfo(np.float32).eps)  # constants.f90:45, epsilon(1.)


def lonlat(p):
    """cart2sph (smeshpack.f90): longitude in [-pi, pi] (0 on the z axis)
    and latitude of points p[..., 3]."""
    p = np.asarray(p, dtype=np.float64)
    x, y, z = p[..., 0], p[..., 1], p[..., 2]
    lon = np.where((x != 0.0) | (y != 0.0), np.arctan2(y, x), 0.0)
    nrm = np.sqrt(x * x + y * y + z * z)
    lat = np.arcsin(z / np.where(nrm > 0, nrm, 1.0))
    return lon, lat


def arclen(p, q):
    """Angle between unit vectors p and q (Renka's ARCLEN, SSRFPACK): from
    d = |p + q|^2, 2 atan(sqrt((4 - d) / d)), without an inverse cosine."""
    s = np.asarray(p, dtype=np.float64) + np.asarray(q, dtype=np.float64)
    d = s[..., 0] * s[..., 0] + s[..., 1] * s[..., 1] + s[..., 2] * s[..., 2]
    with np.errstate(divide="ignore", invalid="ignore"):
        a = 2.0 * np.arctan(np.sqrt((4.0 - d) / d))
    return np.where(d == 0.0, PI, np.where(d >= 4.0, 0.0, a))


def sph2cart(lon, lat):
    c = np.cos(lat)
    return np.stack([c * np.cos(lon), c * np.sin(lon), np.sin(lat)], axis=-1)


def _edge_u(grid: Grid, vlon, vlat):
    """Normal velocity along ed%tg of a (zonal, meridional) field given at
    the edge midpoints."""
    v = convert_vec_sph2cart(vlon, vlat, grid.ed_c)
    return dot3(v, grid.ed_tg)


# ---- case 0 --------------------------------------------------------------
def tc0(grid: Grid):
    lon, lat = lonlat(grid.v_p)
    h = np.cos(lon) * np.cos(grid.v_lat) ** 2
    return h, np.zeros(grid.ne), np.zeros(grid.nv)


# ---- case 1 --------------------------------------------------------------
def tc1(grid: Grid):
    """Cosine bell of height 1000 m and radius a/3 centred at (0, 0) in a
    solid-body rotation of period 12 days."""
    u0 = 2.0 * PI * ERAD / (12.0 * DAY2SEC)
    h0 = 1000.0
    rmax = ERAD / 3.0
    p0 = sph2cart(0.0, 0.0)
    r = ERAD * arclen(grid.v_p, p0)
    h = np.where(r < rmax, (h0 * 0.5) * (1.0 + np.cos(PI * r / rmax)), 0.0)
    u = _edge_u(grid, u0 * np.cos(grid.ed_c_lat), 0.0)
    return h, u, np.zeros(grid.nv)


# ---- case 5 --------------------------------------------------------------
def tc5(grid: Grid):
    """Case-2-like zonal flow (u0 = 20 m/s, h0 = 5960 m) over a cone 2000 m
    high and pi/9 wide centred at (-pi/2, pi/6); h is the free surface minus
    the topography."""
    u0, h0 = 20.0, 5960.0
    h_ct = (ERAD * OMEGA * u0 + (u0 * u0) / 2.0) * GRAVI
    lon0, lat0, rmax = -PI * 0.5, PI / 6.0, PI / 9.0
    lon, _ = lonlat(grid.v_p)
    lat = grid.v_lat
    r = np.sqrt((lon - lon0) ** 2 + (lat - lat0) ** 2)
    bt = np.where(r < rmax, 2000.0 * (1.0 - r / rmax), 0.0)
    h = (h0 - h_ct * np.sin(lat) ** 2) - bt
    u = _edge_u(grid, u0 * np.cos(grid.ed_c_lat), 0.0)
    return h, u, bt


# ---- case 6 --------------------------------------------------------------
TC6_K = 7.848e-6   # K_RH = w, swm.f90:1428-1429
TC6_W = 7.848e-6
TC6_M = 4
TC6_H0 = 8.0e3


def tc6_velocity(lon, lat):
    """(zonal, meridional) velocity of the Rossby-Haurwitz wave; works on
    complex arguments (complex-step derivatives)."""
    m, K, w = TC6_M, TC6_K, TC6_W
    c, s = np.cos(lat), np.sin(lat)
    ul = ERAD * w * c + ERAD * K * c ** (m - 1) * (m * s * s - c * c) * np.cos(m * lon)
    vl = -ERAD * K * m * c ** (m - 1) * s * np.sin(m * lon)
    return ul, vl


def tc6_height(lon, lat):
    """h_tc6 (swm.f90:2392-2413): h0 + a^2/g (A + B cos(m lon) + C cos(2 m
    lon)), A set to 0 within float epsilon of the poles."""
    m, K, w = TC6_M, TC6_K, TC6_W
    c = np.cos(lat)
    with np.errstate(divide="ignore", invalid="ignore"):
        a = (0.5 * w * (2.0 * OMEGA + w) * c ** 2
             + 0.25 * K ** 2 * c ** (m * 2)
             * ((m + 1) * c ** 2 + (2.0 * m ** 2 - m - 2.0) - 2.0 * m ** 2 / (c ** 2)))
    a = np.where(np.abs(np.real(lat)) > PIO2 - EPS, 0.0, a)
    b = 2.0 * ((OMEGA + w) * K / ((m + 1) * (m + 2))) * c ** m \
        * ((m ** 2 + 2.0 * m + 2.0) - (m + 1) ** 2 * c ** 2)
    cc = 0.25 * K ** 2 * c ** (2 * m) * ((m + 1) * c ** 2 - (m + 2))
    return TC6_H0 + GRAVI * (ERAD ** 2) * (a + b * np.cos(m * lon) + cc * np.cos(2.0 * m * lon))


def tc6(grid: Grid):
    elon, elat = lonlat(grid.ed_c)
    ul, vl = tc6_velocity(elon, grid.ed_c_lat)
    u = _edge_u(grid, ul, vl)
    lon, _ = lonlat(grid.v_p)
    h = tc6_height(lon, grid.v_lat)
    return h, u, np.zeros(grid.nv)


def _dd(f, lon, lat, wrt, step=1e-30):
    """Complex-step derivative of f(lon, lat) with respect to lon (wrt=0) or
    lat (wrt=1)."""
    if wrt == 0:
        return np.imag(f(lon + 1j * step, lat + 0j)) / step
    return np.imag(f(lon + 0j, lat + 1j * step)) / step


def tc6_exact_tendency(grid: Grid):
    """Exact (masseq[nv], momeq[ne]) of the case-6 initial state, bt = 0:
    masseq = -div(h v) at the cells; momeq = (-eta k x v - grad(g h + K)) .
    ed%tg at the edge midpoints, with eta = zeta + 2 Omega sin(lat)."""
    def hu(lo, la):
        return tc6_height(lo, la) * tc6_velocity(lo, la)[0]

    def hv_cos(lo, la):
        return tc6_height(lo, la) * tc6_velocity(lo, la)[1] * np.cos(la)

    lon, _ = lonlat(grid.v_p)
    lat = grid.v_lat
    with np.errstate(divide="ignore", invalid="ignore"):
        div = (_dd(hu, lon, lat, 0) + _dd(hv_cos, lon, lat, 1)) / (ERAD * np.cos(lat))
    masseq = -div

    elon, _ = lonlat(grid.ed_c)
    elat = grid.ed_c_lat
    ul, vl = tc6_velocity(elon, elat)

    def vel_u_cos(lo, la):
        return tc6_velocity(lo, la)[0] * np.cos(la)

    def vel_v(lo, la):
        return tc6_velocity(lo, la)[1]

    def bern(lo, la):
        a, b = tc6_velocity(lo, la)
        return GRAV * tc6_height(lo, la) + 0.5 * (a * a + b * b)

    c = np.cos(elat)
    zeta = (_dd(vel_v, elon, elat, 0) - _dd(vel_u_cos, elon, elat, 1)) / (ERAD * c)
    eta = zeta + 2.0 * OMEGA * np.sin(elat)
    # k x (u e_lon + v e_lat) = u e_lat - v e_lon
    mlon = eta * vl - _dd(bern, elon, elat, 0) / (ERAD * c)
    mlat = -eta * ul - _dd(bern, elon, elat, 1) / ERAD
    momeq = _edge_u(grid, mlon, mlat)
    return masseq, momeq


CASES = {0: tc0, 1: tc1, 2: None, 5: tc5, 6: tc6}


def initialize_fields(grid: Grid, testcase: int):
    """(h[nv], u[ne], bt[nv]) of a test case (0, 1, 2, 5 or 6)."""
    if testcase == 2:
        h, u = initialize_fields_tc2(grid)
        return h, u, np.zeros(grid.nv)
    if testcase not in CASES:
        raise ValueError(f"test case {testcase} is not built (cases: {sorted(CASES)})")
    return CASES[testcase](grid)
