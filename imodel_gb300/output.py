"""Text and binary outputs of iModel's shallow-water test driver.

The files ``swm_tests`` writes (src/swm.f90:2754-3152), in the same layout,
so that the reference's plotting scripts (pyscripts/) read runs of this
library unchanged:

* ``swm_errors.txt``                      write_errors      swm.f90:2922-2990
* ``<swmname>_evolution_<grid>.txt``       write_evol_error  swm.f90:2992-3086
* ``<swmname>_mass_energy_<grid>.txt``     write_evol        swm.f90:3088-3152
* ``<name>_<grid>.dat`` field dumps: float32 (lon, lat, value) triples on a
  720 x 1440 pixel-registered lat-lon grid, value of the nearest cell
  (plot_scalarfield, interpack.f90:7376-7510).

Numbers are written with Fortran edit descriptors (``Ew.d``, ``Fw.d``,
``Iw``, ``Aw``) as gfortran prints them.
"""
from __future__ import annotations

import math
import os

import numpy as np

from .mesh import PI, Grid

RAD2DEG = 1.0 / (PI / 180.0)


def fortran_e(x: float, w: int, d: int) -> str:
    """Fortran Ew.d: 0.ddddE+xx, right-justified in w columns."""
    if not math.isfinite(x):
        s = "NaN" if math.isnan(x) else ("-Infinity" if x < 0 else "Infinity")
        return s.rjust(w)
    if x == 0.0:
        body = "0." + "0" * d + "E+00"
        return body.rjust(w)
    m, e = f"{abs(x):.{d - 1}e}".split("e")
    digits = m.replace(".", "")
    exp = int(e) + 1
    ex = f"E{exp:+03d}" if abs(exp) <= 99 else f"{exp:+04d}"
    body = ("-" if x < 0 else "") + "0." + digits + ex
    return body.rjust(w)


def fortran_f(x: float, w: int, d: int) -> str:
    s = f"{x:.{d}f}"
    return s.rjust(w) if len(s) <= w else "*" * w


def fortran_i(k: int, w: int) -> str:
    s = str(int(k))
    return s.rjust(w) if len(s) <= w else "*" * w


def fortran_a(s: str, w: int) -> str:
    return s.rjust(w) if len(s) <= w else s[:w]


def swmname(testcase: int, dt: float, stag: str = "HTC", wrapper: str = "trsk10",
            areamtd: str = "geo") -> str:
    """Run name of swmpars (swm_data.f90:609-689) for the trsk10 path."""
    return f"swm_tc{testcase}_dt{int(round(dt))}_{stag}_{wrapper}_area{areamtd}"


def mean_vdist_deg(grid: Grid) -> float:
    """mesh%meanvdist in degrees (smeshpack.f90:655-690)."""
    return float(np.mean(grid.ed_leng)) * RAD2DEG


_ERR_HEAD = ("       Mesh  TCase    nTime     dt                   TimeDays  "
             "        MaxError_h          RMSError_h            MaxError_u     "
             "   RMSError_u               Mass              Penergy      "
             "     Kenergy             Tenergy             ExtraData                    "
             "                Methods  Grid    ")


def write_errors(datadir: str, grid: Grid, testcase: int, ntime: int, dt: float,
                 time_s: float, errormax_h: float, error2_h: float, errormax_u: float,
                 error2_u: float, error_mass: float, penergy: float, kenergy: float,
                 tenergy: float, tmp: float = 0.0) -> str:
    """Appends one line to swm_errors.txt ('(i12, i4, i10, 11e20.10, a120)')."""
    path = os.path.join(datadir, "swm_errors.txt")
    new = not os.path.exists(path)
    vals = [dt, time_s / 86400.0, errormax_h, error2_h, errormax_u, error2_u, error_mass,
            penergy, kenergy, tenergy, tmp]
    line = (fortran_i(grid.nv, 12) + fortran_i(testcase, 4) + fortran_i(ntime, 10) +
            "".join(fortran_e(v, 20, 10) for v in vals) +
            fortran_a(swmname(testcase, dt) + " " + grid.name, 120))
    with open(path, "a") as f:
        if new:
            f.write(_ERR_HEAD + "\n")
        f.write(line + "\n")
    return path


_EVOL_ERR_HEAD = ("        n        mvdist  tcase       k       nt    "
                  "     dt                 cfl               TimeDays  "
                  "        errormax_h       error2_h               errormax_u     "
                  "   error2_u               errormax_pv       error2_pv            "
                  " mass              Penergy      "
                  "     Kenergy             Tenergy          Availenergy      "
                  "     RMSdiv              maxdiv    "
                  "     max_gradke          tmp        SWMparameters")


def evolution_error_line(grid: Grid, testcase: int, k: int, ntime: int, dt: float, cfl: float,
                         time_s: float, e: dict, tmass: float, pe: float, ke: float, te: float,
                         ae: float, rmsdiv: float, maxdiv: float, max_gradke: float,
                         tmp: float = 0.0) -> str:
    """One line of the evolution file ('(i12, 1f12.4, i4, 2i10, 18e20.10, a100)')."""
    vals = [dt, cfl, time_s / 86400.0, e["errormaxrel_h"], e["error2_h"], e["errormaxrel_u"],
            e["error2_u"], e.get("errormax_pv", 0.0), e.get("error2_pv", 0.0), tmass, pe, ke,
            te, ae, rmsdiv, maxdiv, max_gradke, tmp]
    return (fortran_i(grid.nv, 12) + fortran_f(mean_vdist_deg(grid), 12, 4) +
            fortran_i(testcase, 4) + fortran_i(k, 10) + fortran_i(ntime, 10) +
            "".join(fortran_e(v, 20, 10) for v in vals) +
            fortran_a(swmname(testcase, dt) + "_" + grid.name, 100))


def evolution_path(datadir: str, grid: Grid, testcase: int, dt: float) -> str:
    return os.path.join(datadir, f"{swmname(testcase, dt)}_evolution_{grid.name}.txt")


_EVOL_HEAD = ("        n        mvdist  tcase       k       nt        dt(s)       "
              "          cfl                 time(dys)             mass               Penergy    "
              "          Kenergy            Tenergy            Availenergy           RMSdiv")


def mass_energy_line(grid: Grid, testcase: int, k: int, ntime: int, dt: float, cfl: float,
                     time_s: float, tmass: float, pe: float, ke: float, te: float, ae: float,
                     rmsdiv: float) -> str:
    """One line of the mass/energy file ('(i12, 1f12.4, i4, 2i10, 9e28.16)')."""
    vals = [dt, cfl, time_s / 86400.0, tmass, pe, ke, te, ae, rmsdiv]
    return (fortran_i(grid.nv, 12) + fortran_f(mean_vdist_deg(grid), 12, 4) +
            fortran_i(testcase, 4) + fortran_i(k, 10) + fortran_i(ntime, 10) +
            "".join(fortran_e(v, 28, 16) for v in vals))


def mass_energy_path(datadir: str, grid: Grid, testcase: int, dt: float) -> str:
    return os.path.join(datadir, f"{swmname(testcase, dt)}_mass_energy_{grid.name}.txt")


def open_with_header(path: str, header: str):
    f = open(path, "w")
    f.write(header + "\n")
    return f


def field_dump(path: str, grid: Grid, values, nlat: int = 720, nlon: int = 1440):
    """float32 (lon, lat, value) triples on a pixel-registered lat-lon grid,
    each pixel taking the value of the nearest cell node."""
    from scipy.spatial import cKDTree
    dlat = 180.0 / nlat
    dlon = 360.0 / nlon
    lat = -90.0 + dlat * (np.arange(nlat) + 0.5)
    lon = -180.0 + dlon * (np.arange(nlon) + 0.5)
    LON, LAT = np.meshgrid(lon, lat)
    la, lo = np.deg2rad(LAT.ravel()), np.deg2rad(LON.ravel())
    pts = np.stack([np.cos(la) * np.cos(lo), np.cos(la) * np.sin(lo), np.sin(la)], axis=1)
    _, idx = cKDTree(grid.v_p).query(pts)
    out = np.empty((pts.shape[0], 3), dtype=np.float32)
    out[:, 0] = LON.ravel()
    out[:, 1] = LAT.ravel()
    out[:, 2] = np.asarray(values)[idx]
    out.tofile(path)
    return path


def run_tc2_with_outputs(grid: Grid, dt: float, days: float, datadir: str,
                         precision: str = "fp64", nprints: int = 0):
    """Williamson case 2 with the reference's text outputs: the per-print
    evolution and mass/energy lines and the final error table."""
    from . import swm
    os.makedirs(datadir, exist_ok=True)
    testcase = 2
    h0, u0 = swm.initialize_fields_tc2(grid)
    m = swm.SWM(grid, precision=precision, testcase=testcase)
    ntime = swm.ntime_for(days, dt)
    nprints = nprints if nprints > 0 else ntime
    cfl = 0.0
    try:
        m.set_state(h0, u0)
        d0 = m.diagnostics()
        fe = open_with_header(evolution_path(datadir, grid, testcase, dt), _EVOL_ERR_HEAD)
        fm = open_with_header(mass_energy_path(datadir, grid, testcase, dt), _EVOL_HEAD)
        k = 0
        zero = {"errormaxrel_h": 0.0, "error2_h": 0.0, "errormaxrel_u": 0.0, "error2_u": 0.0}
        fe.write(evolution_error_line(grid, testcase, 0, ntime, dt, cfl, 0.0, zero, d0["mass"],
                                      d0["penergy"], d0["kenergy"], d0["tenergy"],
                                      d0["availenergy"], 0.0, 0.0, 0.0) + "\n")
        fm.write(mass_energy_line(grid, testcase, 0, ntime, dt, cfl, 0.0, d0["mass"],
                                  d0["penergy"], d0["kenergy"], d0["tenergy"],
                                  d0["availenergy"], 0.0) + "\n")
        while k < ntime:
            n = min(nprints, ntime - k)
            m.advance(dt, n)
            k += n
            d = m.diagnostics()
            e = m.errors(h0, u0)
            rel = lambda a, b: (a - b) / b  # noqa: E731
            fe.write(evolution_error_line(
                grid, testcase, k, ntime, dt, cfl, k * dt, e, rel(d["mass"], d0["mass"]),
                rel(d["penergy"], d0["penergy"]), rel(d["kenergy"], d0["kenergy"]),
                rel(d["tenergy"], d0["tenergy"]), rel(d["availenergy"], d0["availenergy"]),
                d["rms_div"], d["max_div"], 0.0) + "\n")
            fm.write(mass_energy_line(
                grid, testcase, k, ntime, dt, cfl, k * dt, rel(d["mass"], d0["mass"]),
                rel(d["penergy"], d0["penergy"]), rel(d["kenergy"], d0["kenergy"]),
                rel(d["tenergy"], d0["tenergy"]), rel(d["availenergy"], d0["availenergy"]),
                d["rms_div"]) + "\n")
        fe.close()
        fm.close()
        write_errors(datadir, grid, testcase, ntime, dt, ntime * dt, e["errormaxrel_h"],
                     e["error2_h"], e["errormaxrel_u"], e["error2_u"],
                     (d["mass"] - d0["mass"]) / d0["mass"],
                     (d["penergy"] - d0["penergy"]) / d0["penergy"],
                     (d["kenergy"] - d0["kenergy"]) / d0["kenergy"],
                     (d["tenergy"] - d0["tenergy"]) / d0["tenergy"])
        h, _ = m.get_state()
        field_dump(os.path.join(datadir, f"{swmname(testcase, dt)}_h_t{ntime}_{grid.name}.dat"),
                   grid, h)
    finally:
        m.close()
