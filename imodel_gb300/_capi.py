"""ctypes mirror of include/imodel_swm.h and include/imodel_mesh.h.

The structures here are field-for-field copies of the C declarations; the
functions load the in-tree shared libraries that ``imodel_gb300._build``
compiles (``imodel_gb300/_lib``).  Loading fails loudly when a library is
missing: there is no fallback implementation of the time step.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(_HERE, "_lib")

c_i32p = ctypes.POINTER(ctypes.c_int32)
c_f64p = ctypes.POINTER(ctypes.c_double)

OK = 0
EINVAL = 1
ECUDA = 2
EBLOWUP = 3
EDIVZERO = 4
ENOMEM = 5
ESTATE = 6
ENODEV = 7
ETOOBIG = 8

FP64 = 0
FP32 = 1
# method wrappers (swm_data.f90:446-507); "dtred" is mtdwrapper "none" with
# coriolis_reconmtd = dtred
SCHEMES = {"trsk10": 0, "pxt16": 1, "gass18": 2, "dtred": 3}

STATUS_NAMES = {
    OK: "OK", EINVAL: "EINVAL", ECUDA: "ECUDA", EBLOWUP: "EBLOWUP",
    EDIVZERO: "EDIVZERO", ENOMEM: "ENOMEM", ESTATE: "ESTATE", ENODEV: "ENODEV",
    ETOOBIG: "ETOOBIG",
}


class Mesh(ctypes.Structure):
    """struct imodel_swm_mesh."""

    _fields_ = [
        ("nv", ctypes.c_int32), ("ne", ctypes.c_int32), ("nt", ctypes.c_int32),
        ("nnb", c_i32p), ("v_nb", c_i32p), ("v_ed", c_i32p), ("v_tr", c_i32p),
        ("hx_ttgout", c_i32p), ("hx_tnrccw", c_i32p),
        ("hx_areag", c_f64p), ("hx_hxtr_area", c_f64p), ("hx_trskw", c_f64p),
        ("v_p", c_f64p), ("v_lat", c_f64p),
        ("ed_v", c_i32p), ("ed_sh", c_i32p), ("ed_leng", c_f64p),
        ("edhx_leng", c_f64p), ("ed_c", c_f64p), ("ed_c_lat", c_f64p),
        ("ed_tg", c_f64p), ("ed_nr", c_f64p),
        ("tr_v", c_i32p), ("tr_ed", c_i32p), ("tr_tg", c_i32p),
        ("tr_areag", c_f64p), ("tr_trhx_area", c_f64p), ("tr_c_lat", c_f64p),
        ("erad", ctypes.c_double), ("grav", ctypes.c_double),
        ("omega", ctypes.c_double),
    ]


class MeshExtra(ctypes.Structure):
    """struct imodel_mesh_extra."""

    _fields_ = [
        ("v_lon", c_f64p), ("ed_c_lon", c_f64p), ("tr_c", c_f64p),
        ("edhx_c", c_f64p), ("edhx_nr", c_f64p), ("edhx_tg", c_f64p),
        ("hx_nr", c_i32p), ("tr_nr", c_i32p),
    ]


class Opts(ctypes.Structure):
    """struct imodel_swm_opts."""

    _fields_ = [
        ("precision", ctypes.c_int32), ("testcase", ctypes.c_int32),
        ("bt", c_f64p), ("h_ref", ctypes.c_double), ("device", ctypes.c_int32),
        ("learned", ctypes.c_int32), ("mlp_weights", ctypes.c_void_p),
        ("mlp_bytes", ctypes.c_size_t), ("drift_bound", ctypes.c_double),
        ("scheme", ctypes.c_int32), ("fsphere", ctypes.c_int32), ("fcte", ctypes.c_double),
        ("error_bound", ctypes.c_double),
    ]


class Diag(ctypes.Structure):
    """struct imodel_swm_diag."""

    _fields_ = [
        ("mass", ctypes.c_double), ("penergy", ctypes.c_double),
        ("kenergy", ctypes.c_double), ("tenergy", ctypes.c_double),
        ("availenergy", ctypes.c_double), ("pot_enstrophy", ctypes.c_double),
        ("rms_div", ctypes.c_double), ("max_div", ctypes.c_double),
        ("learned_active", ctypes.c_int32), ("nan_found", ctypes.c_int32),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


# Every symbol the headers declare, per library (checked by the CPU tests).
MESH_SYMBOLS = [
    "imodel_mesh_build", "imodel_mesh_view", "imodel_mesh_extra_view",
    "imodel_mesh_delaunay_violations", "imodel_mesh_free",
    "imodel_mesh_build_gpu", "imodel_mesh_gpu_last_error",
]
SWM_SYMBOLS = [
    "imodel_swm_create", "imodel_swm_step", "imodel_swm_tendency",
    "imodel_swm_diagnostics", "imodel_swm_errors", "imodel_swm_trsk_tangent",
    "imodel_swm_destroy", "imodel_swm_last_error", "imodel_swm_set_state",
    "imodel_swm_get_state", "imodel_swm_advance", "imodel_swm_profile",
    "imodel_swm_autotune", "imodel_swm_set_tuning", "imodel_swm_set_diffusion",
    "imodel_swm_set_diffusion_fields", "imodel_swm_set_apvm", "imodel_swm_test_fail_alloc",
    "imodel_swm_learned_weights", "imodel_swm_learned_error_proxy",
    "imodel_swm_test_layout_digest",
    "imodel_swm_launch_count",
    "imodel_swm_main_kernel", "imodel_swm_stream", "imodel_swm_weighted_sums_noalloc",
    "imodel_swm_ensemble_create", "imodel_swm_ensemble_set_state",
    "imodel_swm_ensemble_get_state", "imodel_swm_ensemble_advance", "imodel_swm_ensemble_tune",
    "imodel_swm_ensemble_test_stall",
    "imodel_swm_ensemble_destroy", "imodel_swm_ensemble_last_error",
    "imodel_swm_ensemble_stream",
]

MLP_SYMBOLS = [
    "imodel_mlp_create", "imodel_mlp_set_params", "imodel_mlp_get_params",
    "imodel_mlp_forward", "imodel_mlp_grad", "imodel_mlp_load_dataset", "imodel_mlp_train",
    "imodel_mlp_destroy", "imodel_mlp_last_error",
]

MOIST_SYMBOLS = [
    "imodel_moist_create", "imodel_moist_set_state", "imodel_moist_advance",
    "imodel_moist_get_state", "imodel_moist_destroy", "imodel_moist_last_error",
]


class MoistOpts(ctypes.Structure):
    """struct imodel_moist_opts."""

    _fields_ = [("testcase", ctypes.c_int32), ("bt", c_f64p), ("theta", c_f64p),
                ("q0", ctypes.c_double), ("device", ctypes.c_int32),
                ("advection", ctypes.c_int32), ("precision", ctypes.c_int32)]


_libs: dict = {}


def lib_path(name: str) -> str:
    return os.path.join(LIB_DIR, name)


def _load(name: str) -> ctypes.CDLL:
    if name in _libs:
        return _libs[name]
    path = lib_path(name)
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is not built; run imodel_gb300._build.build_all() "
            "(or __graft_entry__.build()) first")
    lib = ctypes.CDLL(path)
    _libs[name] = lib
    return lib


def mesh_lib() -> ctypes.CDLL:
    lib = _load("libimodel_mesh.so")
    if not getattr(lib, "_typed", False):
        lib.imodel_mesh_build.argtypes = [ctypes.c_int32, ctypes.c_int32,
                                          ctypes.c_int32,
                                          ctypes.POINTER(ctypes.c_void_p)]
        lib.imodel_mesh_view.argtypes = [ctypes.c_void_p, ctypes.POINTER(Mesh)]
        lib.imodel_mesh_extra_view.argtypes = [ctypes.c_void_p,
                                               ctypes.POINTER(MeshExtra)]
        lib.imodel_mesh_delaunay_violations.argtypes = [
            ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
            ctypes.POINTER(ctypes.c_double)]
        lib.imodel_mesh_free.argtypes = [ctypes.c_void_p]
        lib.imodel_mesh_free.restype = None
        lib.imodel_mesh_build_gpu.argtypes = [ctypes.c_int32, ctypes.c_int32,
                                              ctypes.c_int32,
                                              ctypes.POINTER(ctypes.c_void_p)]
        lib.imodel_mesh_gpu_last_error.argtypes = []
        lib.imodel_mesh_gpu_last_error.restype = ctypes.c_char_p
        lib._typed = True
    return lib


def swm_lib() -> ctypes.CDLL:
    lib = _load("libimodel_swm.so")
    if not getattr(lib, "_typed", False):
        vp = ctypes.c_void_p
        lib.imodel_swm_create.argtypes = [ctypes.POINTER(Mesh), ctypes.POINTER(Opts),
                                          ctypes.POINTER(vp)]
        lib.imodel_swm_step.argtypes = [vp, c_f64p, c_f64p, ctypes.c_double,
                                        ctypes.c_int32]
        lib.imodel_swm_tendency.argtypes = [vp, c_f64p, c_f64p, c_f64p, c_f64p]
        lib.imodel_swm_diagnostics.argtypes = [vp, ctypes.POINTER(Diag)]
        lib.imodel_swm_errors.argtypes = [vp, c_f64p, c_f64p, c_f64p]
        lib.imodel_swm_trsk_tangent.argtypes = [vp, c_f64p, c_f64p]
        lib.imodel_swm_destroy.argtypes = [vp]
        lib.imodel_swm_last_error.argtypes = [vp]
        lib.imodel_swm_last_error.restype = ctypes.c_char_p
        lib.imodel_swm_set_state.argtypes = [vp, c_f64p, c_f64p]
        lib.imodel_swm_get_state.argtypes = [vp, c_f64p, c_f64p]
        lib.imodel_swm_advance.argtypes = [vp, ctypes.c_double, ctypes.c_int32]
        lib.imodel_swm_set_diffusion.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        lib.imodel_swm_set_apvm.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        lib.imodel_swm_set_diffusion_fields.argtypes = [vp, ctypes.c_void_p, ctypes.c_void_p]
        lib.imodel_swm_profile.argtypes = [vp, ctypes.c_double, ctypes.c_int32, c_f64p]
        lib.imodel_swm_autotune.argtypes = [vp, ctypes.c_double, ctypes.c_int32, c_i32p]
        lib.imodel_swm_set_tuning.argtypes = [vp, c_i32p]
        lib.imodel_swm_launch_count.argtypes = [vp, ctypes.c_int32,
                                                ctypes.POINTER(ctypes.c_int64)]
        lib.imodel_swm_main_kernel.argtypes = [vp]
        lib.imodel_swm_main_kernel.restype = ctypes.c_char_p
        lib.imodel_swm_stream.argtypes = [vp]
        lib.imodel_swm_stream.restype = ctypes.c_void_p
        lib.imodel_swm_weighted_sums_noalloc.argtypes = [vp, vp, ctypes.c_int64, vp, vp]
        lib.imodel_swm_test_fail_alloc.argtypes = [ctypes.c_int32]
        lib.imodel_swm_learned_weights.argtypes = [vp, c_f64p, c_f64p]
        lib.imodel_swm_learned_error_proxy.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
        lib.imodel_swm_test_layout_digest.argtypes = [ctypes.POINTER(Mesh), ctypes.c_int32,
                                                       ctypes.c_int32,
                                                       ctypes.POINTER(ctypes.c_uint64)]
        lib.imodel_swm_ensemble_create.argtypes = [ctypes.POINTER(Mesh), ctypes.c_int32, c_i32p,
                                                   ctypes.c_int32, ctypes.c_int32,
                                                   ctypes.POINTER(vp)]
        lib.imodel_swm_ensemble_set_state.argtypes = [vp, ctypes.c_int32, ctypes.c_int32,
                                                      c_f64p, c_f64p]
        lib.imodel_swm_ensemble_get_state.argtypes = [vp, ctypes.c_int32, ctypes.c_int32,
                                                      c_f64p, c_f64p]
        lib.imodel_swm_ensemble_advance.argtypes = [vp, c_f64p, c_i32p]
        lib.imodel_swm_ensemble_tune.argtypes = [vp, c_f64p, ctypes.c_int32, c_i32p]
        lib.imodel_swm_ensemble_test_stall.argtypes = [vp, ctypes.c_int32, ctypes.c_int64]
        lib.imodel_swm_ensemble_destroy.argtypes = [vp]
        lib.imodel_swm_ensemble_last_error.argtypes = [vp]
        lib.imodel_swm_ensemble_last_error.restype = ctypes.c_char_p
        lib.imodel_swm_ensemble_stream.argtypes = [vp]
        lib.imodel_swm_ensemble_stream.restype = ctypes.c_void_p
        u16p = ctypes.POINTER(ctypes.c_uint16)
        f32p = ctypes.POINTER(ctypes.c_float)
        lib.imodel_mlp_create.argtypes = [ctypes.c_int32, ctypes.POINTER(vp)]
        lib.imodel_mlp_set_params.argtypes = [vp, f32p, ctypes.c_int32]
        lib.imodel_mlp_get_params.argtypes = [vp, f32p, ctypes.c_int32]
        lib.imodel_mlp_forward.argtypes = [vp, u16p, ctypes.c_int64, f32p]
        lib.imodel_mlp_grad.argtypes = [vp, u16p, f32p, f32p, ctypes.c_int64, ctypes.c_uint64,
                                        ctypes.c_int64, f32p, ctypes.POINTER(ctypes.c_double)]
        lib.imodel_mlp_load_dataset.argtypes = [vp, u16p, f32p, f32p, ctypes.c_int64]
        lib.imodel_mlp_train.argtypes = [vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_float,
                                         ctypes.c_uint64, f32p]
        lib.imodel_mlp_destroy.argtypes = [vp]
        lib.imodel_mlp_last_error.argtypes = [vp]
        lib.imodel_mlp_last_error.restype = ctypes.c_char_p
        f64pp = ctypes.POINTER(c_f64p)
        lib.imodel_moist_create.argtypes = [ctypes.POINTER(Mesh), ctypes.POINTER(MoistOpts),
                                            ctypes.POINTER(vp)]
        lib.imodel_moist_set_state.argtypes = [vp, f64pp, c_f64p, c_f64p, c_f64p]
        lib.imodel_moist_advance.argtypes = [vp, ctypes.c_double, ctypes.c_int32]
        lib.imodel_moist_get_state.argtypes = [vp, f64pp]
        lib.imodel_moist_destroy.argtypes = [vp]
        lib.imodel_moist_last_error.argtypes = [vp]
        lib.imodel_moist_last_error.restype = ctypes.c_char_p
        lib._typed = True
    return lib


def as_i32p(a):
    return a.ctypes.data_as(c_i32p)


def as_f64p(a):
    return a.ctypes.data_as(c_f64p)
