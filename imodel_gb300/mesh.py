"""Icosahedral Voronoi/Delaunay grids (Python side of the C++ grid builder).

``meshbuild(level, pos)`` mirrors smeshpack's ``meshbuild`` for
``kind=icos, optm=nopt, hrchy=1`` (src/smeshpack.f90:77-368) and returns a
:class:`Grid` whose numpy arrays are the ``grid_structure`` fields the time
step consumes, 1-based like the Fortran arrays (see include/imodel_swm.h).
The TRSK precomputation of ``initialize_gridprop`` (src/swm.f90:979-992:
kite areas and ``calc_trisk_weights``) is part of the build.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi

ERAD = 6.37122e6       # constants.f90:55
GRAV = 9.80616         # constants.f90:61
OMEGA = 7.292e-5       # constants.f90:67
# constants.f90:31 builds pi from a default-real literal (float32)
PI = 4.0 * float(np.float32(0.78539816339744830961566))
DAY2SEC = 86400.0


def nodes_at_level(level: int) -> int:
    """Number of cells of icosahedral level ``level`` (smeshpack.f90:1531)."""
    return 10 * 4 ** level + 2


_I32 = {"nnb": (1,), "v_nb": (6,), "v_ed": (6,), "v_tr": (6,),
        "hx_ttgout": (6,), "hx_tnrccw": (6,), "ed_v": (2,), "ed_sh": (2,),
        "tr_v": (3,), "tr_ed": (3,), "tr_tg": (3,)}
_F64 = {"hx_areag": (1,), "hx_hxtr_area": (6,), "hx_trskw": (6, 6),
        "v_p": (3,), "v_lat": (1,), "ed_leng": (1,), "edhx_leng": (1,),
        "ed_c": (3,), "ed_c_lat": (1,), "ed_tg": (3,), "ed_nr": (3,),
        "tr_areag": (1,), "tr_trhx_area": (3,), "tr_c_lat": (1,)}
_COUNT = {"nnb": "nv", "v_nb": "nv", "v_ed": "nv", "v_tr": "nv",
          "hx_ttgout": "nv", "hx_tnrccw": "nv", "hx_areag": "nv",
          "hx_hxtr_area": "nv", "hx_trskw": "nv", "v_p": "nv", "v_lat": "nv",
          "ed_v": "ne", "ed_sh": "ne", "ed_leng": "ne", "edhx_leng": "ne",
          "ed_c": "ne", "ed_c_lat": "ne", "ed_tg": "ne", "ed_nr": "ne",
          "tr_v": "nt", "tr_ed": "nt", "tr_tg": "nt", "tr_areag": "nt",
          "tr_trhx_area": "nt", "tr_c_lat": "nt"}
_EXTRA_F64 = {"v_lon": ("nv", (1,)), "ed_c_lon": ("ne", (1,)),
              "tr_c": ("nt", (3,)), "edhx_c": ("ne", (3,)),
              "edhx_nr": ("ne", (3,)), "edhx_tg": ("ne", (3,))}
_EXTRA_I32 = {"hx_nr": ("nv", (6,)), "tr_nr": ("nt", (3,))}


class Grid:
    """A structured grid: numpy copies of the grid_structure arrays.

    Attributes carry the reference names (``nnb``, ``v_ed``, ``hx_trskw`` ...)
    with the shapes of include/imodel_swm.h; ``hx_trskw[c, j, i]`` is the
    reference's ``mesh%hx(c)%trskw(i, j)``.
    """

    def __init__(self, arrays: dict, level: int = -1, pos: str = "eqs",
                 delaunay=(0, 0.0)):
        self.level = level
        self.pos = pos
        self.nv = int(arrays["nnb"].shape[0])
        self.ne = int(arrays["ed_v"].shape[0])
        self.nt = int(arrays["tr_v"].shape[0])
        self.erad, self.grav, self.omega = ERAD, GRAV, OMEGA
        self.delaunay_violations, self.delaunay_margin = delaunay
        for k, v in arrays.items():
            setattr(self, k, v)
        self._struct = None

    @property
    def name(self) -> str:
        return f"icos_{self.pos}_nopt_{self.level}"

    def c_struct(self) -> _capi.Mesh:
        """A ``imodel_swm_mesh`` pointing into this grid's arrays."""
        if self._struct is None:
            m = _capi.Mesh()
            m.nv, m.ne, m.nt = self.nv, self.ne, self.nt
            for k in _I32:
                a = np.ascontiguousarray(getattr(self, k), dtype=np.int32)
                setattr(self, k, a)
                setattr(m, k, _capi.as_i32p(a))
            for k in _F64:
                a = np.ascontiguousarray(getattr(self, k), dtype=np.float64)
                setattr(self, k, a)
                setattr(m, k, _capi.as_f64p(a))
            m.erad, m.grav, m.omega = self.erad, self.grav, self.omega
            self._struct = m
        return self._struct

    # zero-based conveniences -------------------------------------------
    def ed_v0(self):
        return self.ed_v.astype(np.int64) - 1

    def ed_sh0(self):
        return self.ed_sh.astype(np.int64) - 1


class _GridMemory:
    """Owns a grid built by the library; every array of the Grid views its
    memory and holds a reference, so it is freed with the last of them."""

    def __init__(self, lib, handle):
        self.lib, self.handle = lib, handle

    def __del__(self):
        if self.handle:
            self.lib.imodel_mesh_free(self.handle)
            self.handle = None


def _view(ptr, n: int, owner: _GridMemory) -> np.ndarray:
    """A writable numpy view of n elements at the ctypes pointer ptr that
    keeps `owner` alive (no copy: a level-10 grid is about 12 GB)."""
    ctype = ptr._type_
    if n == 0:
        return np.zeros(0, dtype=np.dtype(ctype))
    raw = (ctype * n).from_address(ctypes.cast(ptr, ctypes.c_void_p).value)
    raw._owner = owner
    return np.frombuffer(raw, dtype=np.dtype(ctype))


def meshbuild(level: int, pos: str = "eqs", nthreads: int = 0, device=None) -> Grid:
    """Builds icosahedral grid ``level`` ("eqs" or "pol" base positions).

    With ``device`` (a CUDA device number) the geometry is computed on that
    GPU (imodel_mesh_build_gpu); the numbering is the same, lengths, areas
    and weights agree with the host build to a few units in the last place.
    """
    lib = _capi.mesh_lib()
    handle = ctypes.c_void_p()
    ipos = {"eqs": 0, "pol": 1}[pos]
    if device is None:
        rc = lib.imodel_mesh_build(level, ipos, nthreads, ctypes.byref(handle))
        what = "imodel_mesh_build"
    else:
        rc = lib.imodel_mesh_build_gpu(level, ipos, int(device), ctypes.byref(handle))
        what = "imodel_mesh_build_gpu"
    if rc != 0:
        msg = _capi.STATUS_NAMES.get(rc, rc)
        if device is not None:
            msg = f"{msg} {lib.imodel_mesh_gpu_last_error().decode()}"
        raise RuntimeError(f"{what} failed: {msg}")
    owner = _GridMemory(lib, handle)
    view = _capi.Mesh()
    lib.imodel_mesh_view(handle, ctypes.byref(view))
    extra = _capi.MeshExtra()
    lib.imodel_mesh_extra_view(handle, ctypes.byref(extra))
    n = {"nv": view.nv, "ne": view.ne, "nt": view.nt}
    arrays = {}
    fields = [(k, view, n[_COUNT[k]], shp) for k, shp in list(_I32.items()) + list(_F64.items())]
    fields += [(k, extra, n[c], shp) for k, (c, shp) in
               list(_EXTRA_F64.items()) + list(_EXTRA_I32.items())]
    for k, src, cnt, shp in fields:
        shape = (cnt,) if shp == (1,) else (cnt,) + shp
        arrays[k] = _view(getattr(src, k), int(np.prod(shape)), owner).reshape(shape)
    cnt = ctypes.c_int64()
    margin = ctypes.c_double()
    lib.imodel_mesh_delaunay_violations(handle, ctypes.byref(cnt), ctypes.byref(margin))
    return Grid(arrays, level=level, pos=pos, delaunay=(cnt.value, margin.value))
