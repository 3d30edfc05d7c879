"""Initial states of iModel's other shallow-water test cases on HTC points.

``initialize_fields`` (src/swm.f90:1134-2380) fills h, u and the bottom
topography for a test-case number.  Case 2 lives in ``swm.py``; this module
adds:

* 0 -- time-discretisation check: h = cos(lon) cos^2(lat), u = 0
  (swm.f90:1135-1146);
* 1 -- solid-body rotation of a cosine bell, the advection test (momentum
  equation off; swm.f90:1148-1203);
* 5 -- zonal flow over an isolated conical mountain (Williamson et al.
  1992, case 5; swm.f90:1327-1423);
* 6 -- Rossby-Haurwitz wave of wavenumber 4 (Williamson case 6;
  swm.f90:1426-1620, height ``h_tc6`` at :2392-2413);
* 21, 22, 23 -- the Galewsky et al. (2004) barotropic jet with its height
  perturbation (21), without it (22, a steady balanced jet), and the
  200 m/s jet with the perturbation (23) (swm.f90:1646-1810).

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


# ---- cases 21, 22, 23 -----------------------------------------------------
def galewsky(grid: Grid, testcase: int = 21):
    """Galewsky, Scott and Polvani (2004) barotropic jet, as the reference sets
    it up (swm.f90:1646-1810, after J. Thuburn): the zonal jet u(lat) =
    umax/en exp(1 / ((lat - lat0)(lat - lat1))) between lat0 = pi/7 and
    lat1 = pi/2 - lat0 (case 23: umax 200 m/s, else 80 m/s); the balanced
    height tabulated on 4 floor(sqrt(nv)) latitude intervals by the trapezoid
    rule on d(gh)/dlat = -a u (f + tan(lat) u / a), shifted to a 10 km mean
    depth and interpolated to the cells (cubic Lagrange, linear in the end
    intervals); cases 21 and 23 add the 120 m height bump at (0, pi/4)."""
    u00 = 200.0 if testcase == 23 else 80.0
    lat0 = PI / 7.0
    lat1 = PI / 2.0 - lat0
    en = np.exp(-4.0 / (lat1 - lat0) ** 2)
    umen = u00 / en

    def jet(lat):
        den = (lat - lat0) * (lat - lat1)
        with np.errstate(divide="ignore", over="ignore"):
            return np.where(den < 0.0, umen * np.exp(1.0 / np.where(den < 0.0, den, -1.0)), 0.0)

    # REAL(mesh%nv) is a default (single-precision) real
    nygg = 4 * int(np.floor(np.sqrt(np.float32(grid.nv))))
    dygg = PI / nygg
    hgg = np.zeros(nygg + 1)
    totarea = totvol = 0.0
    for j in range(2, nygg + 1):
        l1 = (j - 2) * dygg - PIO2
        l2 = (j - 1) * dygg - PIO2
        u1, u2 = float(jet(l1)), float(jet(l2))
        u1 = u1 * (2.0 * OMEGA * np.sin(l1) + np.tan(l1) * u1 / ERAD)
        u2 = u2 * (2.0 * OMEGA * np.sin(l2) + np.tan(l2) * u2 / ERAD)
        hgg[j - 1] = hgg[j - 2] - ERAD * 0.5 * (u1 + u2) * dygg
        totarea = totarea + np.cos(l2) * dygg
        totvol = totvol + hgg[j - 1] * np.cos(l2) * dygg
    hgg[nygg] = hgg[nygg - 1]
    totvol = totvol / (totarea * GRAV)
    hgg = (hgg + (1.0e4 - totvol) * GRAV) * GRAVI

    l1 = grid.v_lat + PIO2
    jy = np.floor(l1 / dygg).astype(np.int64) + 1          # 1-based interval
    beta = (l1 - (jy - 1) * dygg) / dygg
    g = lambda k: hgg[np.clip(k - 1, 0, nygg)]            # noqa: E731  hgg(k), 1-based
    lin = (1.0 - beta) * g(jy) + beta * g(jy + 1)
    c1 = -beta * (beta - 1.0) * (beta - 2.0) / 6.0
    c2 = 0.5 * (beta + 1.0) * (beta - 1.0) * (beta - 2.0)
    c3 = -0.5 * (beta + 1.0) * beta * (beta - 2.0)
    c4 = (beta + 1.0) * beta * (beta - 1.0) / 6.0
    cub = c1 * g(jy - 1) + c2 * g(jy) + c3 * g(jy + 1) + c4 * g(jy + 2)
    h = np.where((jy == 1) | (jy == nygg), lin, cub)

    u = _edge_u(grid, jet(grid.ed_c_lat), 0.0)

    if testcase in (21, 23):
        hpert, alpha, bet = 120.0, 1.0 / 3.0, 1.0 / 15.0
        lat2 = 0.5 * PIO2
        lon, _ = lonlat(grid.v_p)
        h = h + hpert * np.cos(grid.v_lat) * np.exp(-(lon / alpha) ** 2) \
            * np.exp(-((lat2 - grid.v_lat) / bet) ** 2)
    return h, u, np.zeros(grid.nv)


# ---- cases 56, 57: Matsuno equatorial waves ------------------------------
MATSUNO_H0 = 30.0
MATSUNO_N = 1
MATSUNO_K = 5.0
MATSUNO_AM = float(np.float32(0.00001))   # a default-real literal


def matsuno_parameters(testcase: int):
    """parameters_matsuno (swm_matsuno.f90): frequency w of the n = 1,
    k = 5 wave -- the largest root of the cubic dispersion relation for the
    inertia-gravity wave (56), the smallest in magnitude, sign flipped, for
    the Rossby wave (57) -- and the coefficients of its Hermite-function
    structure.  The square roots of (n+1)/2 and n/2 are taken in single
    precision, as the reference's real() conversions do."""
    if testcase not in (56, 57):
        raise ValueError("Matsuno cases are 56 (inertia-gravity) and 57 (Rossby)")
    a, g, h0, n = ERAD, GRAV, MATSUNO_H0, MATSUNO_N
    eps = (2.0 * OMEGA * a) ** 2 / (g * h0)
    ks = MATSUNO_K / a
    d0 = 3.0 * (g * h0 * ks * ks + 2.0 * OMEGA * np.sqrt(g * h0) * (2.0 * n + 1.0) / a)
    d4 = -54.0 * OMEGA * g * h0 * ks / a
    w_nk = np.empty(3)
    for j in (1, 2, 3):
        d = np.sqrt(complex(d4 ** 2 - 4.0 * d0 ** 3))
        d = (d + d4) * 0.5
        d = d ** (1.0 / 3.0)
        d = d * np.exp((2.0 * PI * j / 3.0) * 1j)
        w_nk[j - 1] = -np.real(d + d0 / d) / 3.0
    w = w_nk.max() if testcase == 56 else -np.abs(w_nk).min()
    c1 = eps ** 0.25 / a
    c2 = g * h0 * eps ** 0.25 / ((w * w - g * h0 * ks * ks) * a) / 1j
    s1 = float(np.sqrt(np.float32((n + 1.0) * 0.5)))
    s0 = float(np.sqrt(np.float32(n * 0.5)))
    coef = np.array([c1,
                     c2 * (-s1 * (w / np.sqrt(g * h0) + ks)),
                     c2 * (-s0 * (w / np.sqrt(g * h0) - ks)),
                     c2 * (-s1 * (w + np.sqrt(g * h0) * ks)),
                     c2 * (s0 * (w - np.sqrt(g * h0) * ks))], dtype=np.complex128)
    return w, ks, coef


def hermite(x, n: int):
    """Normalised Hermite function without its Gaussian (swm_matsuno.f90,
    Hermite): H_0 = pi^(-1/4), H_(i+1) = x sqrt(2/(i+1)) H_i - sqrt(i/(i+1))
    H_(i-1), the last square root in single precision."""
    hm = np.zeros_like(x)
    hc = np.full_like(x, 1.0 / PI ** 0.25)
    for i in range(n):
        r = float(np.sqrt(np.float32(np.float32(i) / np.float32(i + 1))))
        hm, hc = hc, x * np.sqrt(2.0 / (i + 1)) * hc - r * hm
    return hc


def _matsuno_vbar(lat, coef):
    y = lat * ERAD
    yy = np.real(coef[0]) * y
    gauss = np.exp(-0.5 * yy ** 2)
    n = MATSUNO_N
    return [MATSUNO_AM * hermite(yy, k) * gauss for k in (n - 1, n, n + 1)]


def matsuno_fields(grid: Grid, testcase: int, t: float = 0.0):
    """exact_matsuno (swm_matsuno.f90): the wave's h at the cells and its
    velocity along ed%tg at the edge midpoints at time t (s)."""
    w, ks, coef = matsuno_parameters(testcase)
    vm, v0, vp = _matsuno_vbar(grid.v_lat, coef)
    phase = np.exp((ks * grid.v_lon * ERAD - w * t) * 1j)
    h = np.real((coef[3] * vp + coef[4] * vm) * phase) / GRAV + MATSUNO_H0
    vm, v0, vp = _matsuno_vbar(grid.ed_c_lat, coef)
    phase = np.exp((ks * grid.ed_c_lon * ERAD - w * t) * 1j)
    ue = np.real((coef[1] * vp + coef[2] * vm) * phase)
    ve = np.real(v0 * phase)
    return h, _edge_u(grid, ue, ve)


def matsuno(grid: Grid, testcase: int):
    h, u = matsuno_fields(grid, testcase, 0.0)
    return h, u, np.zeros(grid.nv)


CASES = {0: tc0, 1: tc1, 2: None, 5: tc5, 6: tc6,
         21: galewsky, 22: lambda g: galewsky(g, 22), 23: lambda g: galewsky(g, 23),
         56: lambda g: matsuno(g, 56), 57: lambda g: matsuno(g, 57)}


def initialize_fields(grid: Grid, testcase: int):
    """(h[nv], u[ne], bt[nv]) of a test case (0, 1, 2, 5, 6, 21-23, 56, 57)."""
    if testcase == 2:
        h, u = initialize_fields_tc2(grid)
        return h, u, np.zeros(grid.nv)
    if testcase not in CASES:
        raise ValueError(f"test case {testcase} is not built (cases: {sorted(CASES)})")
    return CASES[testcase](grid)
