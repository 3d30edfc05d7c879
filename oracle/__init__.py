"""CPU oracle of the TRSK shallow-water step (test infrastructure only).

The C++ restatement in ``swm_oracle.cpp`` follows iModel's Fortran
(src/swm.f90, src/swm_operators.f90, src/interpack.f90) loop by loop in
FP64.  Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` use it, as the checker; the library never does.

Parity status: the Fortran reference cannot be compiled here (no Fortran
compiler), so bit parity with its binary is unpinned; the oracle is pinned by
the reference's own known answers instead (TC2 steady state and its analytic
operator values, mimetic identities; see tests/test_oracle_kat.py).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liboracle_swm.so")


def build(force: bool = False) -> str:
    """Compiles the oracle with OpenMP and without FMA contraction."""
    src = os.path.join(HERE, "swm_oracle.cpp")
    hdrs = [os.path.join(HERE, "swm_oracle.h"), os.path.join(ROOT, "include", "imodel_swm.h")]
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not os.path.exists(LIB) or any(
            os.path.getmtime(p) > os.path.getmtime(LIB) for p in [src] + hdrs):
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
               "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), src, "-o", LIB]
        subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        from imodel_gb300._capi import Mesh, Diag
        vp, f64p = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
        L.oracle_create.argtypes = [ctypes.POINTER(Mesh), ctypes.c_int32, f64p, ctypes.c_int32]
        L.oracle_create.restype = vp
        L.oracle_destroy.argtypes = [vp]
        L.oracle_destroy.restype = None
        L.oracle_tendency.argtypes = [vp, f64p, f64p, f64p, f64p]
        L.oracle_rk4.argtypes = [vp, f64p, f64p, f64p, f64p, ctypes.c_double]
        L.oracle_run.argtypes = [vp, f64p, f64p, ctypes.c_double, ctypes.c_int32]
        L.oracle_diagnostics.argtypes = [vp, f64p, f64p, ctypes.POINTER(Diag)]
        L.oracle_error_calc.argtypes = [vp, f64p, f64p, ctypes.c_int32, f64p]
        L.oracle_trsk_tangent.argtypes = [vp, f64p, f64p]
        L.oracle_trsk_weights.argtypes = [ctypes.POINTER(Mesh), f64p]
        L.oracle_tc2.argtypes = [ctypes.POINTER(Mesh), f64p, f64p]
        L.oracle_field.argtypes = [vp, ctypes.c_int32, f64p]
        L.oracle_set_diffusion.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        L.oracle_set_apvm.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        L.oracle_set_scheme.argtypes = [vp, ctypes.c_int32]
        L.oracle_set_fcor.argtypes = [vp, ctypes.c_int32, ctypes.c_double]
        L.oracle_moist_create.argtypes = [ctypes.POINTER(Mesh), ctypes.c_int32, f64p, f64p,
                                          ctypes.c_double, ctypes.c_int32]
        L.oracle_moist_create.restype = vp
        L.oracle_moist_destroy.argtypes = [vp]
        L.oracle_moist_destroy.restype = None
        L.oracle_moist_set_q.argtypes = [vp, f64p, f64p, f64p]
        L.oracle_moist_set_advection.argtypes = [vp, ctypes.c_int32]
        L.oracle_moist_run.argtypes = [vp, ctypes.POINTER(f64p), ctypes.c_double, ctypes.c_int32]
        L.oracle_set_diffusion_fields.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


FIELDS = {"h_ed": (0, "ne"), "uh": (1, "ne"), "eta": (2, "nt"), "h_tr": (3, "nt"),
          "q_tr": (4, "nt"), "q_ed": (5, "ne"), "divuh": (6, "nv"), "ke": (7, "nv"),
          "ghbK": (8, "nv"), "grad_ghbK": (9, "ne"), "uhq_perp": (10, "ne"),
          "divu": (11, "nv"), "zeta": (12, "nt"), "eta_ed": (13, "ne"),
          "lapu": (14, "ne"), "lap_lapu": (15, "ne"), "q_grad_ed": (16, "ne"),
          "h_rhb": (17, "ne"), "vhq_tr": (18, "nt3"), "v_hx": (19, "nv3")}

# method wrappers of swm.par (swm_data.f90:446-507); "dtred" is trsk10 with
# coriolis_reconmtd = dtred (mtdwrapper "none")
SCHEMES = {"trsk10": 0, "pxt16": 1, "gass18": 2, "dtred": 3}


class Oracle:
    """The reference's swm_tests state machine on the CPU, for one grid."""

    def __init__(self, grid, testcase: int = 2, bt=None, nthreads: int = 0, k2: float = 0.0,
                 k4: float = 0.0, pvspar: float = 0.0, dt: float = 0.0, k2_hx=None,
                 k4_hx=None, scheme: str = "trsk10", fsphere: int = 0, fcte: float = 0.0):
        self.grid = grid
        self._mesh = grid.c_struct()
        self._bt = None if bt is None else np.ascontiguousarray(bt, dtype=np.float64)
        n = nthreads if nthreads > 0 else (os.cpu_count() or 1)
        self.nthreads = n
        self._h = lib().oracle_create(ctypes.byref(self._mesh), testcase,
                                      None if self._bt is None else _p(self._bt), n)
        if fsphere:
            if lib().oracle_set_fcor(self._h, fsphere, fcte):
                raise ValueError("fsphere must be 0 or 2")
        if scheme != "trsk10":
            if lib().oracle_set_scheme(self._h, SCHEMES[scheme]):
                raise ValueError(f"bad scheme {scheme!r} (or the mesh lacks ed_nr / ed_c)")
        if k2 or k4:
            if lib().oracle_set_diffusion(self._h, k2, k4):
                raise ValueError("bad diffusion coefficients")
        if k2_hx is not None or k4_hx is not None:
            self._kf = [None if f is None else np.ascontiguousarray(f, dtype=np.float64)
                        for f in (k2_hx, k4_hx)]
            p = [None if f is None else f.ctypes.data for f in self._kf]
            if lib().oracle_set_diffusion_fields(self._h, p[0], p[1]):
                raise ValueError("bad diffusion coefficient fields")
        if pvspar:
            if lib().oracle_set_apvm(self._h, pvspar, dt):
                raise ValueError("bad apvm parameter or time step")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_destroy(self._h)
            self._h = None

    def tendency(self, h, u):
        h = np.ascontiguousarray(h, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        m = np.zeros(self.grid.nv)
        mo = np.zeros(self.grid.ne)
        rc = lib().oracle_tendency(self._h, _p(h), _p(u), _p(m), _p(mo))
        if rc:
            raise RuntimeError(f"oracle tendency status {rc}")
        return m, mo

    def ode_rk4(self, h, u, dt):
        h = np.ascontiguousarray(h, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        hn = np.zeros_like(h)
        un = np.zeros_like(u)
        rc = lib().oracle_rk4(self._h, _p(h), _p(u), _p(hn), _p(un), dt)
        if rc:
            raise RuntimeError(f"oracle rk4 status {rc}")
        return hn, un

    def run(self, h, u, dt, nsteps):
        h = np.array(h, dtype=np.float64)
        u = np.array(u, dtype=np.float64)
        rc = lib().oracle_run(self._h, _p(h), _p(u), dt, nsteps)
        if rc:
            raise RuntimeError(f"oracle run status {rc}")
        return h, u

    def diagnostics(self, h, u):
        from imodel_gb300._capi import Diag
        d = Diag()
        h = np.ascontiguousarray(h, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        lib().oracle_diagnostics(self._h, _p(h), _p(u), ctypes.byref(d))
        return d.as_dict()

    def error_calc(self, f, fref, pos: int):
        out = np.zeros(3)
        f = np.ascontiguousarray(f, dtype=np.float64)
        fref = np.ascontiguousarray(fref, dtype=np.float64)
        lib().oracle_error_calc(self._h, _p(f), _p(fref), pos, _p(out))
        return tuple(out)

    def trsk_tangent(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.zeros(self.grid.ne)
        rc = lib().oracle_trsk_tangent(self._h, _p(u), _p(out))
        if rc:
            raise RuntimeError(f"oracle trsk tangent status {rc}")
        return out

    def field(self, name: str):
        which, cnt = FIELDS[name]
        if cnt.endswith("3"):
            out = np.zeros((getattr(self.grid, cnt[:2]), 3))
        else:
            out = np.zeros(getattr(self.grid, cnt))
        if lib().oracle_field(self._h, which, _p(out)):
            raise RuntimeError(f"oracle field {name!r} not available")
        return out


def trsk_weights(grid):
    out = np.zeros(grid.nv * 36)
    lib().oracle_trsk_weights(ctypes.byref(grid.c_struct()), _p(out))
    return out.reshape(grid.nv, 6, 6)


def tc2(grid):
    h = np.zeros(grid.nv)
    u = np.zeros(grid.ne)
    lib().oracle_tc2(ctypes.byref(grid.c_struct()), _p(h), _p(u))
    return h, u


class MoistOracle:
    """The reference's moist shallow-water model (moist_swm.f90, RK4, advmtd
    "trsk" or "upw1") on the CPU, for one grid and test case; fields as in
    imodel_gb300.moist.moist_fields."""

    FIELDS = ("h", "u", "htheta", "hqv", "hqc", "hqr", "htracer")

    ADVECTION = {"trsk": 0, "upw1": 1}

    def __init__(self, grid, testcase: int, fields: dict, nthreads: int = 0,
                 advection: str = "trsk"):
        self.grid = grid
        self._mesh = grid.c_struct()
        self._bt = np.ascontiguousarray(fields["bt"], dtype=np.float64)
        self._theta = np.ascontiguousarray(fields["theta"], dtype=np.float64)
        n = nthreads if nthreads > 0 else (os.cpu_count() or 1)
        self._h = lib().oracle_moist_create(ctypes.byref(self._mesh), testcase, _p(self._bt),
                                            _p(self._theta), float(fields["q0"]), n)
        if not self._h:
            raise ValueError("moist test case must be 1..5")
        q = [np.ascontiguousarray(fields[k], dtype=np.float64) for k in ("qv", "qc", "qr")]
        lib().oracle_moist_set_q(self._h, _p(q[0]), _p(q[1]), _p(q[2]))
        if advection not in self.ADVECTION or \
                lib().oracle_moist_set_advection(self._h, self.ADVECTION[advection]):
            lib().oracle_moist_destroy(self._h)
            self._h = None
            raise ValueError(f"advection {advection!r}: built are {sorted(self.ADVECTION)}")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().oracle_moist_destroy(self._h)
            self._h = None

    def run(self, state: dict, dt: float, nsteps: int) -> dict:
        ys = [np.array(state[k], dtype=np.float64) for k in self.FIELDS]
        arr = (ctypes.POINTER(ctypes.c_double) * 7)(*[_p(y) for y in ys])
        rc = lib().oracle_moist_run(self._h, arr, dt, nsteps)
        if rc:
            raise RuntimeError(f"oracle moist run status {rc}")
        return dict(zip(self.FIELDS, ys))
