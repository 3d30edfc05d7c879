"""Host side of the GB300 shallow-water step, mirroring iModel's swm module.

The reference drives its shallow-water model from ``swm_tests``
(src/swm.f90:102-380): set up the grid (``initialize_gridprop``), fill the
initial state (``initialize_fields``), then loop ``ode_rk4`` with
diagnostics (``sumf_areas``, ``calc_energies``, ``error_calc``).  This module
keeps those names and their argument meaning on top of the C ABI in
include/imodel_swm.h; every evaluation of the step runs in the CUDA library,
which must be built (``imodel_gb300._build``) -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _capi
from .mesh import DAY2SEC, ERAD, GRAV, OMEGA, PI, Grid

GRAVI = 1.0 / GRAV


class SWMError(RuntimeError):
    """A non-zero status of the C ABI; ``code`` is the IMODEL_SWM_E* value."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_capi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


# ---------------------------------------------------------------------------
# initial states (initialize_fields, src/swm.f90:1043-2380)
# ---------------------------------------------------------------------------
def convert_vec_sph2cart(vlon, vlat, p):
    """smeshpack.f90:4379-4417 for arrays of points p[..., 3]."""
    p = np.asarray(p, dtype=np.float64)
    rho = np.sqrt(p[..., 0] * p[..., 0] + p[..., 1] * p[..., 1])
    with np.errstate(invalid="ignore", divide="ignore"):
        v0 = -(vlon * (p[..., 1] / rho)) - (vlat * p[..., 0] * p[..., 2]) / rho
        v1 = vlon * (p[..., 0] / rho) - (vlat * p[..., 1] * p[..., 2]) / rho
        v2 = vlat * rho
    pole = rho == 0
    v0 = np.where(pole, vlat, v0)
    v1 = np.where(pole, vlon, v1)
    v2 = np.where(pole, 0.0, v2)
    return np.stack([v0, v1, v2], axis=-1)


def dot3(a, b):
    """Fortran dot_product of 3-vectors, summed left to right."""
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def tc2_constants():
    """u0, h0, h_ct, eta_ct of Williamson case 2 (swm.f90:1205-1209)."""
    u0 = 2.0 * PI * ERAD / (12.0 * DAY2SEC)
    h0 = 2.94e4 * GRAVI
    h_ct = (ERAD * OMEGA * u0 + (u0 * u0) / 2.0) * GRAVI
    eta_ct = 2.0 * u0 / ERAD + 2.0 * OMEGA
    return u0, h0, h_ct, eta_ct


def initialize_fields_tc2(grid: Grid):
    """Williamson test case 2 on HTC points (swm.f90:1205-1262).

    Returns (h[nv], u[ne]) in the grid's ordering; u is the normal component
    along ``ed%tg`` at the triangle-edge midpoint ``ed%c``.
    """
    u0, h0, h_ct, _ = tc2_constants()
    s = np.sin(grid.v_lat)
    h = h0 - h_ct * (s * s)
    utmp = u0 * np.cos(grid.ed_c_lat)
    v = convert_vec_sph2cart(utmp, 0.0, grid.ed_c)
    u = dot3(v, grid.ed_tg)
    return h, u


def tc2_exact_operators(grid: Grid):
    """Analytic operator values of case 2 used by the local truncation error
    harness (initialize_fields with test_lterror=1, swm.f90:1221-1290)."""
    u0, h0, h_ct, eta_ct = tc2_constants()
    grad_ct = u0 * eta_ct
    lat_v = grid.v_lat
    lat_e = grid.ed_c_lat
    lat_t = grid.tr_c_lat
    out = {}
    out["ke"] = (u0 * np.cos(lat_v)) ** 2 / 2.0
    out["h_ed"] = h0 - h_ct * np.sin(lat_e) ** 2
    vg = convert_vec_sph2cart(0.0, -grad_ct * np.sin(lat_e) * np.cos(lat_e), grid.ed_c)
    out["grad_ghbK"] = dot3(vg, grid.ed_tg)
    out["q_ed"] = eta_ct * np.sin(lat_e) / out["h_ed"]
    v_ed = convert_vec_sph2cart(u0 * np.cos(lat_e), 0.0, grid.ed_c)
    out["uhq_perp"] = -eta_ct * np.sin(lat_e) * dot3(v_ed, grid.ed_nr)
    out["eta"] = eta_ct * np.sin(lat_t)
    out["h_tr"] = h0 - h_ct * np.sin(lat_t) ** 2
    out["q_tr"] = out["eta"] / out["h_tr"]
    out["divuh"] = np.zeros(grid.nv)
    out["masseq"] = np.zeros(grid.nv)
    out["momeq"] = np.zeros(grid.ne)
    # exact tangential velocity along ed%nr (vecrecon target, HTC)
    out["utg"] = dot3(v_ed, grid.ed_nr)
    return out


# ---------------------------------------------------------------------------
# the GB300 step behind the C ABI
# ---------------------------------------------------------------------------
TUNING_KEYS = ("variant", "bs_tri", "bs_pre", "bs_cell", "bs_edge", "mlp_gather")


class SWM:
    """One grid's shallow-water step on the GPU (trsk10, HTC, geodesic areas).

    precision: "fp64" reproduces the reference's FP64 operation order;
    "fp32" runs FP32 state and operators with FP64 integrals.
    scheme: the method wrapper of swm.par, "trsk10", "pxt16", "gass18", or
    "dtred" (trsk10 with the dtred Coriolis reconstruction).  fsphere = 2
    replaces f = 2 Omega sin(lat) by the constant fcte (the f-sphere of test
    cases 33, 35, 40-42).
    learned_params: the per-step learned correction (FP32); learned_weights:
    network parameters of the learned TRSK weights (imodel_gb300.
    learned_weights), applied once at creation.  drift_bound, error_bound:
    the guard's energy-drift and error-proxy bounds (include/imodel_swm.h).
    """

    def __init__(self, grid: Grid, precision: str = "fp64", testcase: int = 2,
                 bt=None, h_ref: float = 0.0, device: int = 0, learned_params=None,
                 drift_bound: float = 0.0, scheme: str = "trsk10", fsphere: int = 0,
                 fcte: float = 0.0, learned_weights=None, error_bound: float = 0.0):
        self.grid = grid
        self.lib = _capi.swm_lib()
        self.precision = precision
        self._mesh = grid.c_struct()
        opts = _capi.Opts()
        opts.precision = {"fp64": _capi.FP64, "fp32": _capi.FP32}[precision]
        opts.testcase = testcase
        self._bt = None
        if bt is not None:
            self._bt = np.ascontiguousarray(bt, dtype=np.float64)
            opts.bt = _capi.as_f64p(self._bt)
        opts.h_ref = h_ref
        opts.device = device
        opts.scheme = _capi.SCHEMES[scheme]
        self.scheme = scheme
        opts.fsphere = fsphere
        opts.fcte = fcte
        self._mlp = None
        if learned_params is not None and learned_weights is not None:
            raise ValueError("learned_params (per-step network) and learned_weights exclude "
                             "each other")
        if learned_params is not None or learned_weights is not None:
            # learned TRSK correction (network parameters, see imodel_mlp.h):
            # mode 1 the per-step network, mode 2 the learned TRSK weights
            p = learned_params if learned_params is not None else learned_weights
            self._mlp = np.ascontiguousarray(p, dtype=np.float32)
            opts.learned = 1 if learned_params is not None else 2
            opts.mlp_weights = self._mlp.ctypes.data
            opts.mlp_bytes = self._mlp.nbytes
            opts.drift_bound = drift_bound
            opts.error_bound = error_bound
        self._handle = ctypes.c_void_p()
        rc = self.lib.imodel_swm_create(ctypes.byref(self._mesh), ctypes.byref(opts),
                                        ctypes.byref(self._handle))
        if rc != 0:
            msg = self._last_error()
            self.close()
            raise SWMError(rc, msg)

    # -- plumbing --------------------------------------------------------
    def _last_error(self) -> str:
        if not self._handle:
            return ""
        s = self.lib.imodel_swm_last_error(self._handle)
        return s.decode() if s else ""

    def _check(self, rc: int):
        if rc != 0:
            raise SWMError(rc, self._last_error())

    def close(self):
        if getattr(self, "_handle", None):
            self.lib.imodel_swm_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._handle

    # -- reference-facing calls -------------------------------------------
    def tendency(self, h, u):
        """tendency(h, u, masseq, momeq), src/swm.f90:2416."""
        h = np.ascontiguousarray(h, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        masseq = np.empty(self.grid.nv)
        momeq = np.empty(self.grid.ne)
        self._check(self.lib.imodel_swm_tendency(self._handle, _capi.as_f64p(h),
                                                 _capi.as_f64p(u), _capi.as_f64p(masseq),
                                                 _capi.as_f64p(momeq)))
        return masseq, momeq

    def ode_rk4(self, h, u, dt: float, nsteps: int = 1):
        """nsteps of ode_rk4 (src/swm.f90:2600) from host arrays; returns the
        new (h, u)."""
        h = np.array(h, dtype=np.float64)
        u = np.array(u, dtype=np.float64)
        self._check(self.lib.imodel_swm_step(self._handle, _capi.as_f64p(h),
                                             _capi.as_f64p(u), dt, nsteps))
        return h, u

    def set_state(self, h, u):
        h = np.ascontiguousarray(h, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        self._check(self.lib.imodel_swm_set_state(self._handle, _capi.as_f64p(h),
                                                  _capi.as_f64p(u)))

    def get_state(self):
        h = np.empty(self.grid.nv)
        u = np.empty(self.grid.ne)
        self._check(self.lib.imodel_swm_get_state(self._handle, _capi.as_f64p(h),
                                                  _capi.as_f64p(u)))
        return h, u

    def advance(self, dt: float, nsteps: int):
        self._check(self.lib.imodel_swm_advance(self._handle, dt, nsteps))

    def set_diffusion(self, k2: float = 0.0, k4: float = 0.0):
        """Laplacian diffusion K2_max (m^2/s) and hyperdiffusion K4_max
        (m^4/s) of the momentum, constant coefficients (swm.f90:169-205,
        swm_operators.f90:855-975); 0 switches a term off."""
        self._check(self.lib.imodel_swm_set_diffusion(self._handle, k2, k4))

    def set_diffusion_fields(self, k2_hx=None, k4_hx=None):
        """Diffusion / hyperdiffusion with per-cell coefficient fields (nv
        values, the "align" / "diam" branches; see imodel_gb300.difcoef);
        None switches a term off."""
        a = [None if f is None else np.ascontiguousarray(f, dtype=np.float64)
             for f in (k2_hx, k4_hx)]
        for f in a:
            if f is not None and f.shape != (self.grid.nv,):
                raise ValueError("a coefficient field has one value per cell")
        p = [None if f is None else f.ctypes.data for f in a]
        self._check(self.lib.imodel_swm_set_diffusion_fields(self._handle, p[0], p[1]))

    def set_apvm(self, pvspar: float, dt: float):
        """pv_stab = "apvm" (swm_operators.f90:1465-1543) with parameter
        pvspar (0 = off) and the run's time step dt; FP32 handles keep
        their variant (1 and 2 add the edge pre-pass before their cell
        kernel)."""
        self._check(self.lib.imodel_swm_set_apvm(self._handle, pvspar, dt))

    def learned_weights(self):
        """(hxtr_area[nv, 6], trskw[nv, 6, 6]) of a handle created with
        learned_weights: the corrected kite fractions and the TRSK weights
        the step uses (trskw(i, j) at [c, j, i])."""
        R = np.zeros((self.grid.nv, 6))
        w = np.zeros((self.grid.nv, 6, 6))
        self._check(self.lib.imodel_swm_learned_weights(self._handle, _capi.as_f64p(R),
                                                        _capi.as_f64p(w)))
        return R, w

    def learned_error_proxy(self) -> float:
        """The guard's error proxy as last measured (-1 before the first):
        relative L2 difference of the learned and the plain momentum
        tendency on the state of that check."""
        v = ctypes.c_double()
        self._check(self.lib.imodel_swm_learned_error_proxy(self._handle, ctypes.byref(v)))
        return v.value

    def diagnostics(self) -> dict:
        """sumf_areas + calc_energies + RMS divergence of the current state."""
        d = _capi.Diag()
        self._check(self.lib.imodel_swm_diagnostics(self._handle, ctypes.byref(d)))
        return d.as_dict()

    def errors(self, h_ref, u_ref) -> dict:
        """error_calc of h and u against reference fields (swm.f90:3492)."""
        h_ref = np.ascontiguousarray(h_ref, dtype=np.float64)
        u_ref = np.ascontiguousarray(u_ref, dtype=np.float64)
        out = np.zeros(6)
        self._check(self.lib.imodel_swm_errors(self._handle, _capi.as_f64p(h_ref),
                                               _capi.as_f64p(u_ref), _capi.as_f64p(out)))
        return {"errormaxrel_h": out[0], "error2_h": out[1], "errormax_h": out[2],
                "errormaxrel_u": out[3], "error2_u": out[4], "errormax_u": out[5]}

    def trsk_tangent(self, u):
        """vecrecon_trsk_tg at every edge (interpack.f90:3852), along ed%nr."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.empty(self.grid.ne)
        self._check(self.lib.imodel_swm_trsk_tangent(self._handle, _capi.as_f64p(u),
                                                     _capi.as_f64p(out)))
        return out

    KERNELS = ("triangle", "edge_pre", "cell", "edge")

    def profile(self, dt: float, nsteps: int) -> dict:
        """Average ms per launch of the four stage kernels (CUDA events on
        the handle's stream, kernels launched one by one)."""
        out = np.zeros(4)
        self._check(self.lib.imodel_swm_profile(self._handle, dt, nsteps, _capi.as_f64p(out)))
        return dict(zip(self.KERNELS, out.tolist()))

    def autotune(self, dt: float, nsteps: int = 5) -> dict:
        """Times the FP32 fusion variants and block sizes on the current
        state, keeps the fastest, restores the state."""
        c = np.zeros(6, dtype=np.int32)
        self._check(self.lib.imodel_swm_autotune(self._handle, dt, nsteps, _capi.as_i32p(c)))
        return dict(zip(TUNING_KEYS, c.tolist()))

    def set_tuning(self, variant: int = 1, bs_tri: int = 256, bs_pre: int = 256,
                   bs_cell: int = 256, bs_edge: int = 256, mlp_gather: int = 2):
        c = np.array([variant, bs_tri, bs_pre, bs_cell, bs_edge, mlp_gather], dtype=np.int32)
        self._check(self.lib.imodel_swm_set_tuning(self._handle, _capi.as_i32p(c)))

    def launch_count(self, nsteps: int) -> int:
        c = ctypes.c_int64()
        self._check(self.lib.imodel_swm_launch_count(self._handle, nsteps, ctypes.byref(c)))
        return c.value

    def main_kernel(self) -> str:
        return self.lib.imodel_swm_main_kernel(self._handle).decode()

    def stream(self) -> int:
        return self.lib.imodel_swm_stream(self._handle) or 0


class Ensemble:
    """Many FP32 instances on up to 8 grids, advanced by one persistent
    launch (see imodel_swm_ensemble_* in include/imodel_swm.h)."""

    def __init__(self, grids, members, testcase: int = 2, device: int = 0):
        self.grids = list(grids)
        self.members = [int(m) for m in members]
        self.lib = _capi.swm_lib()
        structs = (_capi.Mesh * len(self.grids))()
        for k, g in enumerate(self.grids):
            structs[k] = g.c_struct()
        self._structs = structs
        mem = np.ascontiguousarray(self.members, dtype=np.int32)
        self._handle = ctypes.c_void_p()
        rc = self.lib.imodel_swm_ensemble_create(structs, len(self.grids), _capi.as_i32p(mem),
                                                 testcase, device, ctypes.byref(self._handle))
        if rc != 0:
            msg = self._last_error()
            self.close()
            raise SWMError(rc, msg)

    def _last_error(self):
        if not self._handle:
            return ""
        s = self.lib.imodel_swm_ensemble_last_error(self._handle)
        return s.decode() if s else ""

    def _check(self, rc):
        if rc != 0:
            raise SWMError(rc, self._last_error())

    def close(self):
        if getattr(self, "_handle", None):
            self.lib.imodel_swm_ensemble_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, grid: int, member: int, h, u):
        h = np.ascontiguousarray(h, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        self._check(self.lib.imodel_swm_ensemble_set_state(self._handle, grid, member,
                                                           _capi.as_f64p(h), _capi.as_f64p(u)))

    def get_state(self, grid: int, member: int):
        g = self.grids[grid]
        h = np.empty(g.nv)
        u = np.empty(g.ne)
        self._check(self.lib.imodel_swm_ensemble_get_state(self._handle, grid, member,
                                                           _capi.as_f64p(h), _capi.as_f64p(u)))
        return h, u

    def advance(self, dt, nsteps):
        dt = np.ascontiguousarray(dt, dtype=np.float64)
        ns = np.ascontiguousarray(nsteps, dtype=np.int32)
        self._check(self.lib.imodel_swm_ensemble_advance(self._handle, _capi.as_f64p(dt),
                                                         _capi.as_i32p(ns)))

    def tune(self, dt, nsteps: int = 3) -> dict:
        dt = np.ascontiguousarray(dt, dtype=np.float64)
        c = np.zeros(3, dtype=np.int32)
        self._check(self.lib.imodel_swm_ensemble_tune(self._handle, _capi.as_f64p(dt), nsteps,
                                                      _capi.as_i32p(c)))
        return {"block": int(c[0]), "blocks_per_sm": int(c[1]), "variant": int(c[2])}

    def stream(self) -> int:
        return self.lib.imodel_swm_ensemble_stream(self._handle) or 0


def ntime_for(maxtime_days: float, dt: float) -> int:
    """ntime = ceiling(maxtime/dt) (swm_data.f90:573)."""
    return int(math.ceil(maxtime_days * DAY2SEC / dt))


def swm_tests(grid: Grid, dt: float, days: float, precision: str = "fp64",
              nprints: int = 0, testcase: int = 2):
    """A test case run as swm_tests does (swm.f90:102-380): initial state
    (cases 0, 1, 2, 5, 6; imodel_gb300/testcases.py), ntime RK4 steps on the
    GPU, errors against the reference's h_exact/u_exact -- the initial state,
    which is the exact solution of case 2 at every time and of case 1 after
    whole rotation periods (12 days) -- and mass/energy changes.  Returns a
    dict of the final error-table values."""
    from .testcases import initialize_fields
    h0, u0, bt = initialize_fields(grid, testcase)
    m = SWM(grid, precision=precision, testcase=testcase,
            bt=bt if np.any(bt != 0) else None)
    try:
        m.set_state(h0, u0)
        d0 = m.diagnostics()
        ntime = ntime_for(days, dt)
        done = 0
        chunk = nprints if nprints > 0 else ntime
        while done < ntime:
            k = min(chunk, ntime - done)
            m.advance(dt, k)
            done += k
        d = m.diagnostics()
        e = m.errors(h0, u0)
        def change(k):
            # relative change (absolute where the initial value is 0, as the
            # kinetic energy of case 0)
            return (d[k] - d0[k]) / d0[k] if d0[k] != 0 else d[k] - d0[k]

        e.update({"time_days": ntime * dt / DAY2SEC, "ntime": ntime})
        e.update({f"{k}_change": change(k) for k in ("mass", "penergy", "kenergy", "tenergy")})
        return e
    finally:
        m.close()
