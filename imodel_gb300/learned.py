"""Learned correction of the TRSK tangential-velocity reconstruction.

TRSK reconstructs the velocity component along ``ed%nr`` at an edge from the
normal components of the ~10 edges of its two cells (vecrecon_trsk_tg,
src/interpack.f90:3852-3976); on non-optimised icosahedral grids that
reconstruction is inconsistent (its error does not vanish with resolution)
and imprints the grid on the flow.  A small per-edge MLP predicts the
reconstruction error from local inputs:

* 10 velocities: the stencil normal velocities u_k, each times the TRSK sign
  ttgout_c(j) * tnrccw_c(i_e) (the local edge frame), ordered ccw from the
  edge in cell ed%v(1) (5 slots) then in cell ed%v(2) (5 slots), pentagon
  slots zero; divided by their RMS sigma,
* 14 geometry numbers, centred on their values for a regular hexagonal
  grid and scaled so that BF16 keeps the grid-distortion signal:
  10 (l_e / mean l - 1), 10 (d_e / l_e - 1/sqrt 3), 10 (A_c / (l_e d_e) - 3/2)
  for both cells, and 20 (w_c(i_e, j) - w_reg) for the 10 TRSK weights of the
  slots above, w_reg = r/n - 1/2 being the weight of slot r of a regular
  n-gon.

The network (24 -> 64 -> 64 -> 1, GELU, BF16 weights, FP32 accumulation)
outputs the error divided by sigma, so the correction is linear in the
velocity scale.  Training data are seeded smooth velocity fields (spherical
harmonics, rotational + divergent parts) whose exact tangential component is
known analytically.  This module builds inputs and targets on the host; the
kernels that train and apply the network are in the CUDA library.
"""
from __future__ import annotations

import os

import numpy as np

from . import fields
from .mesh import ERAD, Grid
from .swm import convert_vec_sph2cart, dot3

NVEL = 10
NGEO = 14
NFEAT = NVEL + NGEO
HIDDEN = 64
# bound of the network output (error / sigma) applied in the step
CORR_MAX = 0.5
NPARAM = HIDDEN * NFEAT + HIDDEN + HIDDEN * HIDDEN + HIDDEN + HIDDEN + 1  # 5825


def stencil(grid: Grid):
    """Per edge: the 10 stencil edges (-1 = padding), TRSK signs and weights,
    in the feature order described in the module docstring."""
    ne = grid.ne
    idx = np.full((ne, NVEL), -1, dtype=np.int64)
    sgn = np.zeros((ne, NVEL))
    wts = np.zeros((ne, NVEL))
    v_ed = grid.v_ed.astype(np.int64) - 1
    for side in range(2):
        cells = grid.ed_v[:, side].astype(np.int64) - 1
        n = grid.nnb[cells]
        ed = v_ed[cells]                                   # [ne, 6]
        e_ids = np.arange(ne)
        slot = np.argmax(ed == e_ids[:, None], axis=1)     # i_e in each cell
        tnr = grid.hx_tnrccw[cells, slot]
        for r in range(1, 6):
            valid = r < n
            j = (slot + r) % n
            k = ed[e_ids, j]
            s = grid.hx_ttgout[cells, j] * tnr
            w = grid.hx_trskw[cells, j, slot]              # trskw(i_e, j)
            col = side * 5 + (r - 1)
            idx[valid, col] = k[valid]
            sgn[valid, col] = s[valid]
            wts[valid, col] = w[valid]
    return idx, sgn, wts


def regular_weights(grid: Grid):
    """TRSK weight of each stencil slot on a regular n-gon: r/n - 1/2."""
    wreg = np.zeros((grid.ne, NVEL))
    for side in range(2):
        n = grid.nnb[grid.ed_v[:, side] - 1].astype(np.float64)
        for r in range(1, 6):
            wreg[:, side * 5 + r - 1] = np.where(r < n, r / n - 0.5, 0.0)
    return wreg


def geometry_features(grid: Grid, wts=None):
    """The 14 per-edge geometry inputs [ne, 14] (float64)."""
    if wts is None:
        wts = stencil(grid)[2]
    l = grid.ed_leng
    d = grid.edhx_leng
    c1 = grid.ed_v[:, 0] - 1
    c2 = grid.ed_v[:, 1] - 1
    g = np.empty((grid.ne, NGEO))
    g[:, 0] = 10.0 * (l / l.mean() - 1.0)
    g[:, 1] = 10.0 * (d / l - 1.0 / np.sqrt(3.0))
    g[:, 2] = 10.0 * (grid.hx_areag[c1] / (l * d) - 1.5)
    g[:, 3] = 10.0 * (grid.hx_areag[c2] / (l * d) - 1.5)
    g[:, 4:] = 20.0 * (wts - regular_weights(grid))
    return g


def features(grid: Grid, u, st=None, geo=None):
    """Network inputs [ne, 24] and the velocity scale sigma [ne] for the
    normal velocities u (float64 reference implementation)."""
    if st is None:
        st = stencil(grid)
    idx, sgn, wts = st
    if geo is None:
        geo = geometry_features(grid, wts)
    uv = np.where(idx >= 0, u[np.maximum(idx, 0)], 0.0) * sgn
    sigma = np.sqrt(np.mean(uv * uv, axis=1)) + 1e-30
    x = np.empty((grid.ne, NFEAT))
    x[:, :NVEL] = uv / sigma[:, None]
    x[:, NVEL:] = geo
    return x, sigma


def velocity_sample(grid: Grid, lmax: int = 48, seed: int = 0, chi_fraction: float = 0.5,
                    exponent: float = -2.0, umax: float = 40.0):
    """Seeded smooth velocity: normal components u (along ed%tg) and the exact
    tangential components (along ed%nr) at the HTC edge points."""
    a, b = fields.random_coeffs(lmax, seed, exponent)
    sp = fields.Spectral(a, b)
    elon = np.arctan2(grid.ed_c[:, 1], grid.ed_c[:, 0])
    elat = grid.ed_c_lat
    cosl = np.maximum(np.cos(elat), 1e-12)
    psi_lat, psi_lon = sp.eval_grad(elon, elat)
    ulon = -psi_lat / ERAD
    ulat = psi_lon / (ERAD * cosl)
    if chi_fraction > 0:
        ac, bc = fields.random_coeffs(lmax, seed + 7919, exponent)
        sc = fields.Spectral(ac, bc)
        chi_lat, chi_lon = sc.eval_grad(elon, elat)
        dl = chi_lon / (ERAD * cosl)
        dp = chi_lat / ERAD
        k = chi_fraction * np.sqrt(ulon ** 2 + ulat ** 2).max() / np.sqrt(dl ** 2 + dp ** 2).max()
        ulon = ulon + k * dl
        ulat = ulat + k * dp
    scale = umax / np.sqrt(ulon ** 2 + ulat ** 2).max()
    v = convert_vec_sph2cart(ulon * scale, ulat * scale, grid.ed_c)
    return dot3(v, grid.ed_tg), dot3(v, grid.ed_nr)


def init_params(seed: int = 0):
    """Uniform Glorot initial parameters (layout of include/imodel_mlp.h),
    zero biases."""
    rng = np.random.default_rng(seed)
    a1 = np.sqrt(6.0 / (NFEAT + HIDDEN))
    a2 = np.sqrt(6.0 / (HIDDEN + HIDDEN))
    a3 = np.sqrt(6.0 / (HIDDEN + 1))
    return np.concatenate([
        rng.uniform(-a1, a1, HIDDEN * NFEAT), np.zeros(HIDDEN),
        rng.uniform(-a2, a2, HIDDEN * HIDDEN), np.zeros(HIDDEN),
        rng.uniform(-a3, a3, HIDDEN), np.zeros(1)]).astype(np.float32)


TRAINED_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                            "trsk_mlp_l7.npy")


def trained_params(path: str = TRAINED_PATH):
    """Parameters trained by imodel_gb300.train_learned on icosahedral level 7
    (256 seeded fields, degree <= 48); None when the file is absent."""
    if not os.path.exists(path):
        return None
    p = np.load(path).astype(np.float32)
    if p.shape != (NPARAM,):
        raise ValueError(f"{path}: {p.shape} parameters, expected ({NPARAM},)")
    return p


def to_bf16_bits(a):
    """float -> BF16 bit patterns (nearest, ties to even) as uint16."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    return (((b + 0x7FFF + ((b >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


class Mlp:
    """The network on the GPU (include/imodel_mlp.h)."""

    NPARAM = 5825

    def __init__(self, device: int = 0, params=None):
        import ctypes
        from . import _capi
        self._ct = ctypes
        self._capi = _capi
        self.lib = _capi.swm_lib()
        self._h = ctypes.c_void_p()
        rc = self.lib.imodel_mlp_create(device, ctypes.byref(self._h))
        if rc != 0:
            msg = self.lib.imodel_mlp_last_error(self._h)
            self.close()
            raise RuntimeError(f"imodel_mlp_create: {rc} {msg}")
        if params is not None:
            self.set_params(params)

    def _check(self, rc):
        if rc != 0:
            msg = self.lib.imodel_mlp_last_error(self._h)
            raise RuntimeError(f"imodel_mlp: status {rc}: {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "_h", None):
            self.lib.imodel_mlp_destroy(self._h)
            self._h = self._ct.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _f32p(self, a):
        return a.ctypes.data_as(self._ct.POINTER(self._ct.c_float))

    def _u16p(self, a):
        return a.ctypes.data_as(self._ct.POINTER(self._ct.c_uint16))

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(self.lib.imodel_mlp_set_params(self._h, self._f32p(p), p.size))

    def get_params(self):
        p = np.empty(self.NPARAM, dtype=np.float32)
        self._check(self.lib.imodel_mlp_get_params(self._h, self._f32p(p), p.size))
        return p

    def forward(self, xbits):
        xbits = np.ascontiguousarray(xbits, dtype=np.uint16)
        n = xbits.shape[0]
        y = np.empty(n, dtype=np.float32)
        self._check(self.lib.imodel_mlp_forward(self._h, self._u16p(xbits), n, self._f32p(y)))
        return y

    def grad(self, xbits, t, w=None, batch=None, seed=0):
        xbits = np.ascontiguousarray(xbits, dtype=np.uint16)
        t = np.ascontiguousarray(t, dtype=np.float32)
        wp = None
        if w is not None:
            w = np.ascontiguousarray(w, dtype=np.float32)
            wp = self._f32p(w)
        n = xbits.shape[0]
        g = np.empty(self.NPARAM, dtype=np.float32)
        loss = self._ct.c_double()
        self._check(self.lib.imodel_mlp_grad(self._h, self._u16p(xbits), self._f32p(t), wp, n,
                                             seed, batch or n, self._f32p(g),
                                             self._ct.byref(loss)))
        return loss.value, g

    def load_dataset(self, xbits, t, w=None):
        xbits = np.ascontiguousarray(xbits, dtype=np.uint16)
        t = np.ascontiguousarray(t, dtype=np.float32)
        wp = None
        if w is not None:
            self._w = np.ascontiguousarray(w, dtype=np.float32)
            wp = self._f32p(self._w)
        self._check(self.lib.imodel_mlp_load_dataset(self._h, self._u16p(xbits), self._f32p(t),
                                                     wp, xbits.shape[0]))

    def train(self, steps, batch=65536, lr=1e-3, seed=1):
        losses = np.empty(steps, dtype=np.float32)
        self._check(self.lib.imodel_mlp_train(self._h, steps, batch, lr, seed,
                                              self._f32p(losses)))
        return losses


def training_set(grid: Grid, seeds, lmax: int = 48, chi_fraction: float = 0.5,
                 mixtures: int = 0, mix_seed: int = 0):
    """Inputs (BF16 bits [n, 24]), normalised targets (error / sigma) and
    sample weights sigma^2 / mean(sigma^2) of TRSK's tangential
    reconstruction for seeded fields on one grid.  With these weights the
    loss is the mean squared error of the tangential velocity itself, so
    near-stagnation edges (small sigma, where the stencil does not determine
    the error) do not dominate the fit.

    mixtures > 0 adds that many fields formed as random Gaussian combinations
    of the sampled ones: a Gaussian mixture of random spherical-harmonic fields
    is again such a field, and both the TRSK reconstruction and the exact
    tangential component are linear in the velocity, so these samples are
    exact and cost no spectral work."""
    st = stencil(grid)
    geo = geometry_features(grid, st[2])
    base = [velocity_sample(grid, lmax=lmax, seed=s, chi_fraction=chi_fraction) for s in seeds]
    fields_uv = list(base)
    if mixtures > 0:
        rng = np.random.default_rng(mix_seed)
        U = np.stack([b[0] for b in base])
        UT = np.stack([b[1] for b in base])
        for _ in range(mixtures):
            a = rng.standard_normal(len(base)) / np.sqrt(len(base))
            fields_uv.append((a @ U, a @ UT))
    xs, ts, ws = [], [], []
    for u, ut in fields_uv:
        utg = trsk_tangent_np(grid, u, st)
        x, sigma = features(grid, u, st, geo)
        xs.append(to_bf16_bits(x))
        ts.append(((ut - utg) / sigma).astype(np.float32))
        ws.append((sigma * sigma / np.mean(sigma * sigma)).astype(np.float32))
    return np.concatenate(xs), np.concatenate(ts), np.concatenate(ws)


def corrected_tangent(grid: Grid, mlp: Mlp, u, st=None):
    """TRSK tangential velocity plus the network's predicted error, clipped
    to +-CORR_MAX sigma as in the step."""
    if st is None:
        st = stencil(grid)
    utg = trsk_tangent_np(grid, u, st)
    x, sigma = features(grid, u, st)
    y = np.clip(mlp.forward(to_bf16_bits(x)).astype(np.float64), -CORR_MAX, CORR_MAX)
    return utg + sigma * y


def trsk_tangent_np(grid: Grid, u, st=None):
    """vecrecon_trsk_tg (var%pos == 6) in numpy, from the stencil arrays."""
    if st is None:
        st = stencil(grid)
    idx, sgn, wts = st
    uk = np.where(idx >= 0, u[np.maximum(idx, 0)], 0.0)
    d = np.where(idx >= 0, grid.edhx_leng[np.maximum(idx, 0)], 0.0)
    return -np.sum(uk * d * wts * sgn, axis=1) / grid.ed_leng
