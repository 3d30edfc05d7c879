"""Seeded synthetic initial states for the shallow-water step.

The reference's ``initialize_fields`` (src/swm.f90:1043-2380) only holds
analytic test cases; the balanced random states below are new and follow the
generator the benchmark configurations describe:

* streamfunction psi = sum over real spherical harmonics of degree 1..lmax
  with N(0,1) coefficients times l**p (p = -2 for an l^-2 coefficient
  spectrum; p = -3 gives an l^-3 kinetic-energy spectrum),
* u = k x grad(psi) (optionally plus grad(chi) for a divergent part), scaled
  so that the largest wind speed at the velocity points equals ``umax``,
* h from linear balance  g lap(h) = div(f grad(psi)),  mean g h = gh0,
* optional Gaussian mountains; the fluid depth is then h - b so that the
  free surface h + b stays balanced.

Spectral work: fully normalised associated Legendre functions by the
standard three-term recurrences, a Gauss-Legendre grid for the one
projection the balance equation needs, and cubic splines in latitude of the
zonal Fourier coefficients for evaluation at millions of grid points.
"""
from __future__ import annotations

import numpy as np
from scipy.interpolate import CubicSpline

from .mesh import ERAD, GRAV, OMEGA, Grid
from .swm import convert_vec_sph2cart, dot3


# ---------------------------------------------------------------------------
def legendre_m(m: int, lmax: int, mu: np.ndarray) -> np.ndarray:
    """Fully normalised P_lm(mu) for l = m..lmax (rows), points mu (cols)."""
    mu = np.asarray(mu, dtype=np.float64)
    cs = np.sqrt(np.maximum(0.0, 1.0 - mu * mu))
    out = np.zeros((lmax - m + 1, mu.size))
    pmm = np.ones_like(mu) * np.sqrt(1.0 / (4.0 * np.pi))
    for k in range(1, m + 1):
        pmm = -np.sqrt((2.0 * k + 1.0) / (2.0 * k)) * cs * pmm
    out[0] = pmm
    if lmax == m:
        return out
    p1 = np.sqrt(2.0 * m + 3.0) * mu * pmm
    out[1] = p1
    p0 = pmm
    for l in range(m + 2, lmax + 1):
        a = np.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
        b = np.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
        p2 = a * (mu * p1 - b * p0)
        out[l - m] = p2
        p0, p1 = p1, p2
    return out


def random_coeffs(lmax: int, seed: int, exponent: float = -2.0):
    """a[l, m] (cos) and b[l, m] (sin) coefficients, N(0,1) * l**exponent."""
    rng = np.random.default_rng(seed)
    a = np.zeros((lmax + 1, lmax + 1))
    b = np.zeros((lmax + 1, lmax + 1))
    for l in range(1, lmax + 1):
        s = float(l) ** exponent
        a[l, : l + 1] = rng.standard_normal(l + 1) * s
        b[l, 1: l + 1] = rng.standard_normal(l) * s
    return a, b


class Spectral:
    """Synthesis of sum_lm (a_lm cos m lon + b_lm sin m lon) P_lm(sin lat) at
    arbitrary points through latitude splines of the zonal coefficients."""

    def __init__(self, a: np.ndarray, b: np.ndarray, ntab: int = 0):
        self.lmax = a.shape[0] - 1
        L = self.lmax
        ntab = ntab or max(2048, 16 * L)
        self.phi = np.linspace(-np.pi / 2, np.pi / 2, ntab)
        mu = np.sin(self.phi)
        A = np.zeros((ntab, L + 1))
        B = np.zeros((ntab, L + 1))
        for m in range(L + 1):
            P = legendre_m(m, L, mu)
            A[:, m] = a[m:, m] @ P
            B[:, m] = b[m:, m] @ P
        self.splA = CubicSpline(self.phi, A, axis=0)
        self.splB = CubicSpline(self.phi, B, axis=0)

    def eval(self, lon, lat, dlat=False, dlon=False, chunk=0):
        """Field (or its latitude / longitude derivative) at points."""
        chunk = chunk or max(4096, (1 << 24) // (self.lmax + 1))
        lon = np.asarray(lon, dtype=np.float64)
        lat = np.asarray(lat, dtype=np.float64)
        out = np.empty(lon.size)
        m = np.arange(self.lmax + 1, dtype=np.float64)
        for s in range(0, lon.size, chunk):
            la, lo = lat[s:s + chunk], lon[s:s + chunk]
            nu = 1 if dlat else 0
            Am = self.splA(la, nu)
            Bm = self.splB(la, nu)
            ml = np.outer(lo, m)
            c, sn = np.cos(ml), np.sin(ml)
            if dlon:
                out[s:s + chunk] = np.sum(m * (-Am * sn + Bm * c), axis=1)
            else:
                out[s:s + chunk] = np.sum(Am * c + Bm * sn, axis=1)
        return out


    def eval_grad(self, lon, lat, chunk=262144):
        """(d/dlat, d/dlon) of the field at points, in one pass."""
        lon = np.asarray(lon, dtype=np.float64)
        lat = np.asarray(lat, dtype=np.float64)
        flat = np.empty(lon.size)
        flon = np.empty(lon.size)
        m = np.arange(self.lmax + 1, dtype=np.float64)
        for s in range(0, lon.size, chunk):
            la, lo = lat[s:s + chunk], lon[s:s + chunk]
            Am, Bm = self.splA(la), self.splB(la)
            dAm, dBm = self.splA(la, 1), self.splB(la, 1)
            ml = np.outer(lo, m)
            c, sn = np.cos(ml), np.sin(ml)
            flat[s:s + chunk] = np.sum(dAm * c + dBm * sn, axis=1)
            flon[s:s + chunk] = np.sum(m * (Bm * c - Am * sn), axis=1)
        return flat, flon


def gauss_grid(lmax: int):
    nlat = lmax + 3
    x, w = np.polynomial.legendre.leggauss(nlat)
    nlon = 2 * lmax + 6
    lon = 2 * np.pi * np.arange(nlon) / nlon
    return np.arcsin(x), w, lon


def synth_grid(a, b, lat, lon):
    """Exact synthesis (and d/dlat) on a lat x lon grid."""
    L = a.shape[0] - 1
    mu = np.sin(lat)
    cs = np.cos(lat)
    f = np.zeros((lat.size, lon.size))
    fphi = np.zeros_like(f)
    for m in range(L + 1):
        P = legendre_m(m, L + 1, mu)         # l = m..L+1
        l = np.arange(m, L + 1)
        Pl = P[: L - m + 1]
        # dP_lm/dphi = [ -l mu P_lm + c_lm P_{l-1,m} ] / cos(phi)
        Plm1 = np.zeros_like(Pl)
        if L - m >= 1:
            Plm1[1:] = P[: L - m]
        c = np.sqrt((2.0 * l + 1.0) * (l * l - m * m) / np.maximum(2.0 * l - 1.0, 1.0))
        dP = (-l[:, None] * mu[None, :] * Pl + c[:, None] * Plm1) / cs[None, :]
        Am, Bm = a[m:, m] @ Pl, b[m:, m] @ Pl
        dAm, dBm = a[m:, m] @ dP, b[m:, m] @ dP
        cm, sm = np.cos(m * lon), np.sin(m * lon)
        f += np.outer(Am, cm) + np.outer(Bm, sm)
        fphi += np.outer(dAm, cm) + np.outer(dBm, sm)
    return f, fphi


def analyse_grid(f, lat, w, lon, lmax):
    """Spherical-harmonic coefficients of f on a Gauss grid (up to lmax)."""
    nlon = lon.size
    a = np.zeros((lmax + 1, lmax + 1))
    b = np.zeros((lmax + 1, lmax + 1))
    mu = np.sin(lat)
    for m in range(lmax + 1):
        cm = np.cos(m * lon) @ f.T * (2 * np.pi / nlon)
        sm = np.sin(m * lon) @ f.T * (2 * np.pi / nlon)
        P = legendre_m(m, lmax, mu)
        # int P_lm^2 dmu * (2pi or pi)
        norm = (P * P) @ w * (2 * np.pi if m == 0 else np.pi)
        a[m:, m] = (P @ (w * cm)) / norm
        if m > 0:
            b[m:, m] = (P @ (w * sm)) / norm
    return a, b


def spectral_eval(a, b, lon, lat, mode: str = "f"):
    """Synthesis at points: mode "f" (field), "dlat" or "dlon" (derivatives)."""
    return Spectral(a, b).eval(lon, lat, dlat=mode == "dlat", dlon=mode == "dlon")


def _eval_chunk(args):
    a, b, lon, lat, mode = args
    return spectral_eval(a, b, lon, lat, mode)


class PoolEvaluator:
    """spectral_eval split over a process pool by points (the same values as
    the serial evaluation: every point is computed independently)."""

    def __init__(self, pool, chunk: int = 1 << 20):
        self.pool = pool
        self.chunk = chunk

    def __call__(self, a, b, lon, lat, mode="f"):
        lon = np.asarray(lon, dtype=np.float64)
        lat = np.asarray(lat, dtype=np.float64)
        jobs = [(a, b, lon[s:s + self.chunk], lat[s:s + self.chunk], mode)
                for s in range(0, lon.size, self.chunk)]
        return np.concatenate(self.pool.map(_eval_chunk, jobs)) if jobs else np.empty(0)


def balanced_state(grid: Grid, lmax: int = 64, seed: int = 0, exponent: float = -2.0,
                   umax: float = 40.0, gh0: float = 2.94e4, chi_fraction: float = 0.0,
                   bt=None, evaluator=None):
    """Seeded balanced (h, u) on the grid; see the module docstring.

    chi_fraction > 0 adds a divergent part grad(chi) whose coefficients are
    drawn with the same spectrum (seed + 1) and scaled to that fraction of
    the rotational part; the balance equation uses psi only.
    """
    ev = evaluator or spectral_eval
    a, b = random_coeffs(lmax, seed, exponent)
    elon = np.arctan2(grid.ed_c[:, 1], grid.ed_c[:, 0])
    elat = grid.ed_c_lat
    cosl = np.maximum(np.cos(elat), 1e-12)
    # u = k x grad psi : (u_lon, u_lat) = (-dpsi/dphi / a, dpsi/dlon / (a cos))
    ulon = -ev(a, b, elon, elat, "dlat") / ERAD
    ulat = ev(a, b, elon, elat, "dlon") / (ERAD * cosl)
    if chi_fraction > 0:
        ac, bc = random_coeffs(lmax, seed + 1, exponent)
        dlon_c = ev(ac, bc, elon, elat, "dlon") / (ERAD * cosl)
        dlat_c = ev(ac, bc, elon, elat, "dlat") / ERAD
        rot = np.sqrt(ulon ** 2 + ulat ** 2).max()
        div = np.sqrt(dlon_c ** 2 + dlat_c ** 2).max()
        k = chi_fraction * rot / max(div, 1e-300)
        ulon = ulon + k * dlon_c
        ulat = ulat + k * dlat_c
    speed = np.sqrt(ulon ** 2 + ulat ** 2)
    scale = umax / speed.max()
    v = convert_vec_sph2cart(ulon * scale, ulat * scale, grid.ed_c)
    u = dot3(v, grid.ed_tg)

    # linear balance: g lap h = div(f grad psi) = f lap psi + (2 Omega cos / a^2) dpsi/dphi
    glat, gw, glon = gauss_grid(lmax)
    psi, psi_phi = synth_grid(a, b, glat, glon)
    lap_a = a * 0.0
    lap_b = b * 0.0
    for l in range(lmax + 1):
        lap_a[l] = -l * (l + 1) * a[l] / ERAD ** 2
        lap_b[l] = -l * (l + 1) * b[l] / ERAD ** 2
    lap, _ = synth_grid(lap_a, lap_b, glat, glon)
    f = 2 * OMEGA * np.sin(glat)[:, None]
    rhs = f * lap + (2 * OMEGA * np.cos(glat)[:, None] / ERAD ** 2) * psi_phi
    ra, rb = analyse_grid(rhs, glat, gw, glon, lmax + 1)
    ha = np.zeros_like(ra)
    hb = np.zeros_like(rb)
    for l in range(1, lmax + 2):
        ha[l] = -ERAD ** 2 * ra[l] / (GRAV * l * (l + 1))
        hb[l] = -ERAD ** 2 * rb[l] / (GRAV * l * (l + 1))
    vlon = np.arctan2(grid.v_p[:, 1], grid.v_p[:, 0])
    h = gh0 / GRAV + scale * ev(ha, hb, vlon, grid.v_lat, "f")
    if bt is not None:
        h = h - bt
    return h, u


def gaussian_mountains(grid: Grid, n: int = 4, seed: int = 0, hmin=500.0, hmax=2000.0,
                       rmin_deg=5.0, rmax_deg=20.0):
    """Bottom topography: n Gaussian mountains, heights U(hmin, hmax) m,
    radii U(rmin, rmax) degrees, centres uniform on the sphere (seeded)."""
    rng = np.random.default_rng(seed)
    bt = np.zeros(grid.nv)
    p = grid.v_p
    for _ in range(n):
        z = rng.uniform(-1, 1)
        lon = rng.uniform(-np.pi, np.pi)
        r = np.sqrt(1 - z * z)
        c = np.array([r * np.cos(lon), r * np.sin(lon), z])
        height = rng.uniform(hmin, hmax)
        radius = np.deg2rad(rng.uniform(rmin_deg, rmax_deg))
        d = np.arccos(np.clip(p @ c, -1.0, 1.0))
        bt += height * np.exp(-(d / radius) ** 2)
    return bt
