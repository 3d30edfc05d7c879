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
  200 m/s jet with the perturbation (23) (swm.f90:1646-1810); 52 and 53 the
  same jet in the southern hemisphere, without and with a perturbation;
* 32-35 -- the Hollingsworth-instability cases: a thin layer over a bottom
  carrying case 2's balanced height (swm.f90:1918-2068);
* 40-43 -- localised steady states on an f-sphere, two of them rotated
  (swm.f90:2070-2371);
* 51 -- case 5's flow as a thin layer over a Gaussian hill (:1380-1398);
* 56, 57 -- Matsuno's equatorial waves.

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
DEG2RAD = PI / 180.0                   # constants.f90, pi/180._r8
EPS = float(np.finfo(np.float32).eps)  # constants.f90:45, epsilon(1.)
HOLLGW = 2.0                           # swm.par's Hollingsworth layer depth (par/swm.par:29)


def ipow(x, n: int):
    """x**n for an integer n as the Fortran run time evaluates it: square
    and multiply, low bits first (not pow(), whose rounding differs)."""
    x = np.asarray(x, dtype=np.float64)
    result = np.ones_like(x)
    base = x.copy()
    u = int(n)
    while True:
        if u & 1:
            result = result * base
        u >>= 1
        if not u:
            break
        base = base * base
    return result


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
    if testcase in (52, 53):
        # the jet in the southern hemisphere between 5 and 45 degrees south
        u00, lat0, lat1 = 80.0, -5.0 * DEG2RAD, -45.0 * DEG2RAD
    else:
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

    if testcase in (21, 23, 53):
        hpert, alpha, bet = 120.0, 1.0 / 3.0, 1.0 / 15.0
        lat2 = -25.0 * DEG2RAD if testcase == 53 else 0.5 * PIO2
        lon, _ = lonlat(grid.v_p)
        if testcase == 53:
            lon = lon + 120.0 * DEG2RAD
        h = h + hpert * np.cos(grid.v_lat) * np.exp(-(lon / alpha) ** 2) \
            * np.exp(-((lat2 - grid.v_lat) / bet) ** 2)
    return h, u, np.zeros(grid.nv)


# ---- case 51 ----------------------------------------------------------------
def tc51(grid: Grid, hollgw: float = HOLLGW):
    """Case 5's zonal flow as a thin layer (the Hollingsworth depth) over a
    bottom that carries the balanced case-5 height plus a 20 m Gaussian hill
    at (-pi/2, pi/6) (swm.f90:1380-1398); the layer thins by the hill's
    height so that the free surface stays balanced."""
    u0, h0 = 20.0, 5960.0
    h_ct = (ERAD * OMEGA * u0 + (u0 * u0) / 2.0) * GRAVI
    lon0, lat0, rmax = -PI * 0.5, PI / 6.0, PI / 9.0
    p0 = sph2cart(lon0, lat0)
    d = grid.v_p - p0
    r = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
    rmaxc = 2 * (1 - np.cos(rmax))
    c04 = float(np.float32(0.4))   # -0.4 is a default-real literal
    hill = 20.0 * np.exp(-c04 * r ** 2 / rmaxc ** 2)
    bt = (h0 - h_ct * np.sin(grid.v_lat) ** 2) + hill
    h = hollgw - hill
    u = _edge_u(grid, u0 * np.cos(grid.ed_c_lat), 0.0)
    return h, u, bt


# ---- cases 32-35: the Hollingsworth instability ---------------------------
def hollingsworth(grid: Grid, testcase: int = 32, hollgw: float = HOLLGW):
    """A thin layer of depth hollgw riding on a bottom that carries case 2's
    balanced height (swm.f90:1918-2068): 32 and 34 in the rotating frame,
    33 and 35 on an f = 0 sphere (f-sphere, fcte = 0) with the matching
    balance (u0^2/2 only).  34 and 35 start from the same states as 32 and
    33.  Their time loop's linear analysis (swm.f90:251-281: a forcing, a
    perturbation of cell 18, and a rescaling of the departure to 1e-6 of u)
    is not built: at the first step the forcing cancels the departure in u
    to rounding -- exactly, on the grids tried -- and the rescaling factor
    1e-6 / error2_u is then infinite."""
    if testcase not in (32, 33, 34, 35):
        raise ValueError("Hollingsworth cases are 32-35")
    if not hollgw > EPS:
        raise ValueError("the Hollingsworth cases need a positive layer depth")
    u0 = 2.0 * PI * ERAD / (12.0 * DAY2SEC)
    h0 = 2.94e4 * GRAVI
    if testcase in (33, 35):
        h_ct = ((u0 * u0) / 2.0) * GRAVI
    else:
        h_ct = (ERAD * OMEGA * u0 + (u0 * u0) / 2.0) * GRAVI
    bt = h0 - h_ct * np.sin(grid.v_lat) ** 2
    # fsphere = 2 subtracts (erad / grav) fcte sin(lat), with fcte = 0
    h = np.full(grid.nv, float(hollgw))
    u = _edge_u(grid, u0 * np.cos(grid.ed_c_lat), 0.0)
    return h, u, bt


# ---- cases 40-43: localised steady states ---------------------------------
def _rotation(lon0: float, lat0: float):
    """Rmat of swm.f90:2146-2156: takes (lon0, lat0) to the north pole."""
    R = np.zeros((3, 3))
    R[0, 0] = np.sin(lat0) * np.cos(lon0)
    R[0, 1] = np.sin(lat0) * np.sin(lon0)
    R[0, 2] = -np.cos(lat0)
    R[1, 0] = -np.sin(lon0)
    R[1, 1] = np.cos(lon0)
    R[2, 0] = np.cos(lat0) * np.cos(lon0)
    R[2, 1] = np.cos(lat0) * np.sin(lon0)
    R[2, 2] = np.sin(lat0)
    return R


def _matvec(R, p):
    """matmul(R, p) for points p[..., 3], each component summed in order."""
    p = np.asarray(p, dtype=np.float64)
    out = np.empty_like(p)
    for i in range(3):
        s = R[i, 0] * p[..., 0]
        s = s + R[i, 1] * p[..., 1]
        s = s + R[i, 2] * p[..., 2]
        out[..., i] = s
    return out


def localised(grid: Grid, testcase: int = 40):
    """Steady localised states on an f-sphere (swm.f90:2070-2331):

    * 40 -- h = h0 (2 - sin(lat)^n), u = u0 sin(lat)^k cos(lat), k = 120,
      n = 2k + 2, h0 = 10^4 / g, u0 = sqrt(n h0 g), f = 0;
    * 41 -- the same with h0 = 10^5 / g, rotated so that its peak sits at
      (1, 3) degrees;
    * 42 -- k = 160 with f = 1.4584e-4 s^-1, rotated: the northern cap in
      cyclogeostrophic balance u^2 + F u + C = 0, the rest at rest;
    * 43 -- a 20 m/s easterly equatorial jet exp(-50 lat^2) over h = 100 m
      (not balanced: the reference's "play toy")."""
    if testcase == 43:
        umen = -20.0 / 1.0
        u = _edge_u(grid, umen * np.exp(-(grid.ed_c_lat - 0.0) ** 2 * 50.0), 0.0)
        return np.full(grid.nv, 100.0), u, np.zeros(grid.nv)
    if testcase == 40:
        h0, k = 10000 * GRAVI, 120
    elif testcase == 41:
        h0, k = 100000 * GRAVI, 120
    elif testcase == 42:
        h0, k = 100000 * GRAVI, 160
    else:
        raise ValueError("localised cases are 40-43")
    n = k * 2 + 2
    u0 = np.sqrt(n * h0 * GRAV)
    if testcase == 40:
        h = h0 * (2 - ipow(np.sin(grid.v_lat), n))
        lat = grid.ed_c_lat
        u = _edge_u(grid, u0 * ipow(np.sin(lat), k) * np.cos(lat), 0.0)
        return h, u, np.zeros(grid.nv)
    R = _rotation(1 * DEG2RAD, 3 * DEG2RAD)
    _, vlat = lonlat(_matvec(R, grid.v_p))
    if testcase == 41:
        h = h0 * (2 - ipow(np.sin(vlat), n))
    else:
        h = np.where(vlat > 0, h0 * (2 - ipow(np.sin(vlat), n)), 2.0 * h0)
    pe = _matvec(R, grid.ed_c)
    _, elat = lonlat(pe)
    if testcase == 41:
        ut = u0 * ipow(np.sin(elat), k) * np.cos(elat)
    else:
        fcte = 1.4584e-4
        with np.errstate(divide="ignore", invalid="ignore"):
            F = np.where(np.abs(elat) > EPS, ERAD * fcte * np.cos(elat) / np.sin(elat), 0.0)
        C = -GRAV * h0 * n * ipow(np.sin(elat), n - 2) * ipow(np.cos(elat), 2)
        with np.errstate(invalid="ignore"):
            ut = np.where(elat > 0, (-F + np.sqrt(F * F - 4 * C)) / 2, 0.0)
    v = convert_vec_sph2cart(ut, 0.0, pe)
    v = _matvec(R.T, v)
    return h, dot3(v, grid.ed_tg), np.zeros(grid.nv)


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
         32: hollingsworth, 33: lambda g: hollingsworth(g, 33),
         34: lambda g: hollingsworth(g, 34), 35: lambda g: hollingsworth(g, 35),
         40: localised, 41: lambda g: localised(g, 41), 42: lambda g: localised(g, 42),
         43: lambda g: localised(g, 43), 51: tc51,
         52: lambda g: galewsky(g, 52), 53: lambda g: galewsky(g, 53),
         56: lambda g: matsuno(g, 56), 57: lambda g: matsuno(g, 57)}

# cases whose vort_tr runs on an f-sphere (fsphere = 2, constant fcte)
F_SPHERE = {33: 0.0, 35: 0.0, 40: 0.0, 41: 0.0, 42: 1.4584e-4}

# cases that need input data the reference does not ship: 24 reads a
# day-5 ENDGame state from its output directory (swm.f90:1812-1916), 60 the
# ETOPO elevation data of the Andes (refinter.f90:381-469); 11 and 12 are
# the linearised equations of the normal-mode analysis, not a time step
UNAVAILABLE = {24: "needs a day-5 ENDGame GLW state file",
               60: "needs the ETOPO elevation data",
               11: "linearised normal-mode equations", 12: "linearised normal-mode equations"}


def case_options(testcase: int) -> dict:
    """Keyword options of swm.SWM and oracle.Oracle a test case needs
    (testcase number for the momentum switch; the f-sphere)."""
    opts = {"testcase": testcase}
    if testcase in F_SPHERE:
        opts.update(fsphere=2, fcte=F_SPHERE[testcase])
    return opts


def initialize_fields(grid: Grid, testcase: int):
    """(h[nv], u[ne], bt[nv]) of a test case (see CASES)."""
    if testcase == 2:
        h, u = initialize_fields_tc2(grid)
        return h, u, np.zeros(grid.nv)
    if testcase in UNAVAILABLE:
        raise ValueError(f"test case {testcase}: {UNAVAILABLE[testcase]}")
    if testcase not in CASES:
        raise ValueError(f"test case {testcase} is not built (cases: {sorted(CASES)})")
    return CASES[testcase](grid)
