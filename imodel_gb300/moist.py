"""The moist shallow-water model of iModel (src/moist_swm.f90) on the GPU.

Beside h and u the model carries five cell tracers in flux form -- h theta
(potential temperature), h qv, h qc, h qr (vapour, cloud, rain) and a
passive h tracer -- advected by the same C-grid flux as the mass equation
(advmtd = "trsk": div_hx(u * scalar_hx2ed(q)), highorder.f90:4901-4983) or
by first-order upwind fluxes (advmtd = "upw1", :5094-5139), and
the sources of moist_swm.f90:1278-1353: a thermal momentum source
g/2 grad(h^2 theta) / h_e + g theta_e grad(b) added to the shallow-water
momentum tendency, and condensation, evaporation and precipitation between
the water species.  Time stepping is the model's classic RK4
(ode_rk4_moist_swm, :1819-2011); theta, as the sources read it, keeps its
initial value (the RK4 path never updates it), and qv, qc, qr are hq / h
after each step.

``moist_fields`` restates the initial states of test cases 1-5
(initialize_moist_swm_fields, moist_swm.f90:643-1139).  ``Moist`` is the GPU
handle (include/imodel_moist.h): FP64 in the reference's operation order,
or FP32.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from .mesh import DAY2SEC, ERAD, GRAV, OMEGA, PI, Grid
from .swm import SWMError, convert_vec_sph2cart, dot3

GRAVI = 1.0 / GRAV
DEG2RAD = PI / 180.0
PIO2 = PI / 2.0
FIELDS = ("h", "u", "htheta", "hqv", "hqc", "hqr", "htracer")


def qsat(T, H, B, q0):
    """qsat (moist_swm.f90:618-622): q0 exp(20 T) / ((H + B) g)."""
    return q0 * np.exp(20.0 * T) / ((H + B) * GRAV)


def _f_quad(f1, f2, f3, lat):
    """F_quad (moist_swm.f90:630-635): the quadratic in latitude through f1,
    f2, f3 at -pi/2, 0, pi/2."""
    f = lat * (lat - PIO2) * f1 - 2.0 * (lat + PIO2) * (lat - PIO2) * f2 + lat * (lat + PIO2) * f3
    return f * 2.0 / (PI * PI)


def _edge_u(grid: Grid, ulon, vlat):
    v = convert_vec_sph2cart(ulon, vlat, grid.ed_c)
    return dot3(v, grid.ed_tg)


def _tracer(grid: Grid):
    """1 exp(-5 |p - p0|^2) around (0, 0) (the Gaussian hill of cases 1-3),
    p from the cell's longitude and latitude (sph2cart), as the reference
    forms it."""
    lon, lat = grid.v_lon, grid.v_lat
    p = np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], axis=1)
    d = p - np.array([1.0, 0.0, 0.0])
    nrm = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
    return 1.0 * np.exp(-5.0 * (nrm * nrm))


def moist_fields(grid: Grid, testcase: int) -> dict:
    """Initial fields of moist test case 1 (tracer advection by solid-body
    rotation), 2 (a steady balanced moist flow), 3 (moist flow over a
    cone), 4 or 5 (the moist Galewsky jet, northern or southern
    hemisphere): h, u, bt, theta, qv, qc, qr, the flux-form tracers and
    q0."""
    nv = grid.nv
    lon = grid.v_lon
    lat = grid.v_lat
    z = np.zeros(nv)
    if testcase == 1:
        h = np.ones(nv)
        theta, qv, qc, qr, bt = z.copy(), z.copy(), z.copy(), z.copy(), z.copy()
        u0 = 2.0 * PI * ERAD / (12.0 * DAY2SEC)
        u = _edge_u(grid, u0 * np.cos(grid.ed_c_lat), 0.0)
        q0 = 0.0
    elif testcase == 2:
        u0 = 2.0 * PI * ERAD / (12.0 * DAY2SEC)
        phi0 = 3.0 * 10 ** 4
        w = OMEGA * ERAD * u0 + u0 * u0 * 0.5
        sigma = w / 10.0
        temp0 = phi0 * phi0 / 300.0
        xsi = 0.0
        sinn, coss = np.sin(lat), np.cos(lat)
        h = (phi0 - (w + sigma) * sinn ** 2) * GRAVI
        bt = z.copy()
        theta = temp0 + sigma * (coss ** 2) * ((w + sigma) * (coss ** 2) + (phi0 - w - sigma) * 2.0)
        theta = theta / (phi0 ** 2 + ((w + sigma) ** 2) * sinn ** 4
                         - 2.0 * phi0 * (w + sigma) * sinn ** 2)
        qv = (1.0 - xsi) * qsat(theta, h, bt, 1.0)
        qc, qr = z.copy(), z.copy()
        u = _edge_u(grid, u0 * np.cos(grid.ed_c_lat), 0.0)
        q0 = 0.02 / qv.max()
    elif testcase == 3:
        u0, h0 = 20.0, 2000.0
        phi0 = 5960.0 * GRAV
        w = OMEGA * ERAD * u0 + u0 * u0 * 0.5
        xsi, mu1, mu2 = 0.001, 0.05, 0.98
        theta_sp, theta_eq, theta_np = -40.0 / 300.0, 30.0 / 300.0, -20.0 / 300.0
        rmax = PI / 9.0
        lon0 = PI * 0.5 + 30.0 * DEG2RAD
        lat0 = PI / 6.0
        sinn, coss = np.sin(lat), np.cos(lat)
        h = (phi0 - w * sinn ** 2) * GRAVI
        r = np.sqrt((lon - lon0) ** 2 + (lat - lat0) ** 2)
        bt = np.where(r < rmax, 2000.0 * (1.0 - r / rmax), 0.0)
        h = h - bt
        lons = lon + PI + PI + 30.0 * DEG2RAD
        theta = _f_quad(theta_sp, (1.0 - mu1) * theta_eq, theta_np, lat) \
            + mu1 * theta_eq * np.cos(lat) * np.sin(lons)
        qv = mu2 * qsat(theta, h, bt, 1.0)
        qc, qr = z.copy(), z.copy()
        alpha = 0.0
        elon, elat = grid.ed_c_lon, grid.ed_c_lat
        ut = u0 * (np.cos(elat) * np.cos(alpha) + np.cos(elon) * np.sin(elat) * np.sin(alpha))
        vt = -u0 * (np.sin(elon) * np.sin(alpha))
        u = _edge_u(grid, ut, vt)
        q0 = 0.02 / qv.max()
        del h0, xsi
    elif testcase in (4, 5):
        # the moist Galewsky jet (moist_swm.f90:955-1130): the barotropic jet
        # and its tabulated balanced height of swm.f90's cases 22 (jet
        # between pi/7 and 5 pi/14, case 4) and 52 (between 5 and 45 degrees
        # south, case 5), a 120 m bump centred 0.93 pi east (case 4: 120
        # degrees less) at latitude pi/4 (case 4) or -25 degrees (case 5),
        # theta quadratic in latitude and qv at 98 % of saturation
        from .testcases import galewsky
        mu1, mu2 = 0.00002, 0.98
        theta_sp, theta_eq, theta_np = -40.0 / 300.0, 30.0 / 300.0, -20.0 / 300.0
        h, u, bt = galewsky(grid, 22 if testcase == 4 else 52)
        hpert, alpha, beta = 120.0, 1.0 / 3.0, 1.0 / 15.0
        lat2 = 0.5 * PIO2 if testcase == 4 else -25.0 * DEG2RAD
        l1 = lon - 0.93 * PI
        if testcase == 4:
            l1 = l1 + 120.0 * DEG2RAD
        e1 = np.exp(-(l1 / alpha) ** 2)
        e2 = np.exp(-((lat2 - lat) / beta) ** 2)
        h = h + hpert * np.cos(lat) * e1 * e2
        theta = theta_sp * lat * (lat + PIO2) - (1.0 - mu1) * theta_eq * (lat + PIO2) * (lat - PIO2) \
            + theta_np * lat * (lat - PIO2)
        qv = mu2 * qsat(theta, h, bt, 1.0)
        qc, qr = z.copy(), z.copy()
        q0 = 0.02 / qv.max()
    else:
        raise ValueError("moist test cases built: 1, 2, 3, 4, 5")
    # h qv is formed before the q0 scaling, then both are scaled
    hqv = h * qv
    if testcase >= 2:
        qv = q0 * qv
        hqv = q0 * hqv
    # cases 4 and 5 set no tracer (the reference leaves h tracer as
    # allocated; neither case advects it)
    tracer = _tracer(grid) if testcase <= 3 else z.copy()
    return {"h": h, "u": u, "bt": bt, "theta": theta, "qv": qv, "qc": qc, "qr": qr, "q0": q0,
            "htheta": h * theta, "hqv": hqv, "hqc": h * qc, "hqr": h * qr,
            "htracer": tracer * h, "tracer": tracer}


class Moist:
    """The moist shallow-water model on the GPU (include/imodel_moist.h):
    one grid, one test case, FP64 in the reference's operation order or
    FP32; the tracers advected with advmtd "trsk" (centred) or "upw1"
    (first-order upwind, highorder.f90:5094-5139)."""

    ADVECTION = {"trsk": 0, "upw1": 1}
    PRECISION = {"fp64": 0, "fp32": 1}

    def __init__(self, grid: Grid, testcase: int, fields: dict, device: int = 0,
                 advection: str = "trsk", precision: str = "fp64"):
        self.grid = grid
        self.lib = _capi.swm_lib()
        self._mesh = grid.c_struct()
        self._bt = np.ascontiguousarray(fields["bt"], dtype=np.float64)
        self._theta = np.ascontiguousarray(fields["theta"], dtype=np.float64)
        o = _capi.MoistOpts()
        o.testcase = testcase
        o.bt = _capi.as_f64p(self._bt)
        o.theta = _capi.as_f64p(self._theta)
        o.q0 = float(fields["q0"])
        o.device = device
        if advection not in self.ADVECTION:
            raise ValueError(f"advection {advection!r}: built are {sorted(self.ADVECTION)}")
        o.advection = self.ADVECTION[advection]
        if precision not in self.PRECISION:
            raise ValueError(f"precision {precision!r}: built are {sorted(self.PRECISION)}")
        o.precision = self.PRECISION[precision]
        self._handle = ctypes.c_void_p()
        rc = self.lib.imodel_moist_create(ctypes.byref(self._mesh), ctypes.byref(o),
                                          ctypes.byref(self._handle))
        if rc != 0:
            msg = self._last_error()
            self.close()
            raise SWMError(rc, msg)

    def _last_error(self):
        m = self.lib.imodel_moist_last_error(self._handle)
        return m.decode() if m else ""

    def _check(self, rc):
        if rc != 0:
            raise SWMError(rc, self._last_error())

    def close(self):
        if getattr(self, "_handle", None):
            self.lib.imodel_moist_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, state: dict):
        self._in = [np.ascontiguousarray(state[k], dtype=np.float64) for k in FIELDS]
        q = [np.ascontiguousarray(state[k], dtype=np.float64) for k in ("qv", "qc", "qr")]
        arr = (_capi.c_f64p * 7)(*[_capi.as_f64p(a) for a in self._in])
        self._check(self.lib.imodel_moist_set_state(self._handle, arr, *[_capi.as_f64p(a)
                                                                        for a in q]))

    def advance(self, dt: float, nsteps: int):
        self._check(self.lib.imodel_moist_advance(self._handle, dt, nsteps))

    def get_state(self) -> dict:
        out = [np.zeros(self.grid.ne if k == "u" else self.grid.nv) for k in FIELDS]
        arr = (_capi.c_f64p * 7)(*[_capi.as_f64p(a) for a in out])
        self._check(self.lib.imodel_moist_get_state(self._handle, arr))
        return dict(zip(FIELDS, out))
