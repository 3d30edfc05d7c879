"""Learned TRSK weights: a network that corrects the kite fractions TRSK
builds its weights from.

TRSK's tangential reconstruction (vecrecon_trsk_tg, src/interpack.f90:
3852-3976) and Coriolis term (coriolis_ed, src/swm_operators.f90:1283-1308)
use the weights w_c(i, j) = sum_{k=i}^{j-1} R_c(k) - 1/2 of each cell c
(calc_trisk_weights, interpack.f90:3978-4098), where R_c(k) is the fraction
of the cell covered by its k-th kite (hx%hxtr_area).  Any R_c that sums to
one gives weights with TRSK's structure -- antisymmetric, so the Coriolis
term does no work, and compatible with steady geostrophic modes -- and the
kite areas are only one such choice.  On non-optimised icosahedral grids
they are not the most accurate one: the reconstruction error does not
vanish with resolution.

Here a small network (24 -> 64 -> 64 -> 1, GELU, BF16 weights, FP32
accumulation: the tensor-core network of include/imodel_mlp.h) predicts a
correction dR_c(k) of every kite fraction from local geometry (features
below).  The corrections are projected to sum zero per cell and the weights
rebuilt from R + dR: the scheme keeps TRSK's conservation properties by
construction, and the network runs once, when a handle is created -- a step
costs what a plain TRSK step costs.

Training data are made by the method itself: seeded smooth velocity fields
with an exact tangential component (learned.velocity_sample) give, through a
sparse least-squares fit, the kite-fraction corrections that minimise TRSK's
reconstruction error on one grid (``lsq_targets``); the network regresses
them from the geometry with the library's own BF16 training kernels
(``imodel_gb300/train_learned_weights.py``), so that it applies to grids it
was not fitted on.

Features of cell c (n sides, generator p, area A) and kite slot j (the kite
in triangle v%tr(j), between edges v%ed(j) and v%ed(j+1)), all FP64 then
rounded to BF16:

  0-5   10 (R_c(j + dj) - 1/n) for dj = 0, -1, 1, -2, 2, 3 (cyclic)
  6     1 for a pentagon, else 0
  7-8   10 (o . t_j) / sqrt(A), 10 (o . (p x t_j)) / sqrt(A): o is the mean
        of the cell's Voronoi vertices (triangle circumcentres) minus its
        projection on p, t_j the unit tangent from p towards the vertex of
        triangle j
  9-10  10 (d_e / mean d - 1) for the Voronoi edges e = v%ed(j), v%ed(j+1)
  11-12 10 (l_e / mean l - 1) for the same edges' triangle-edge lengths
  13    10 (r_j / mean r - 1), r_j the tangent distance from p to vertex j
  14-23 zero

The same features are computed by the library (swm_layout.cpp,
build_kite_inputs) for imodel_swm_create with opts.learned = 2.
"""
from __future__ import annotations

import os

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as sla

from . import learned
from .mesh import Grid

NFEAT = 24
OUT_SCALE = 0.1   # dR = OUT_SCALE * network output
TRAINED_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                            "trsk_kite_mlp.npy")


def trained_params(path: str = TRAINED_PATH):
    """Parameters trained by imodel_gb300.train_learned_weights; None when
    the file is absent."""
    if not os.path.exists(path):
        return None
    p = np.load(path).astype(np.float32)
    if p.shape != (learned.NPARAM,):
        raise ValueError(f"{path}: {p.shape} parameters, expected ({learned.NPARAM},)")
    return p


def circumcentres(grid: Grid):
    """tr%c%p: the unit normal of each triangle's vertex plane, on the
    vertices' side (the spherical circumcentre)."""
    p = grid.v_p[grid.tr_v - 1]
    a = p[:, 1] - p[:, 0]
    b = p[:, 2] - p[:, 0]
    x = np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1], a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                  a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], axis=1)
    side = np.sum(x * (p[:, 0] + p[:, 1] + p[:, 2]), axis=1)
    nrm = np.sqrt(np.sum(x * x, axis=1)) * np.where(side < 0, -1.0, 1.0)
    return x / nrm[:, None]


def _tangent(v, p):
    return v - np.sum(v * p, axis=-1, keepdims=True) * p


def kite_inputs(grid: Grid):
    """(x[n, 24] float32, cell[n], slot[n]) for every kite slot of every
    cell, slot-major (all slot-0 kites, then slot 1, ...)."""
    nv = grid.nv
    n = grid.nnb.astype(np.int64)
    R = grid.hx_hxtr_area.reshape(nv, 6)
    P = grid.v_p
    sA = np.sqrt(grid.hx_areag)
    cc = circumcentres(grid)
    ved = grid.v_ed.astype(np.int64) - 1
    vtr = grid.v_tr.astype(np.int64) - 1
    mask = np.arange(6)[None, :] < n[:, None]
    T = cc[np.where(mask, vtr, 0)]                       # [nv, 6, 3]
    V = np.zeros((nv, 3))
    for m in range(6):
        V = V + np.where(mask[:, m:m + 1], T[:, m], 0.0)
    V = V / n[:, None]
    O = _tangent(V, P)
    d = grid.edhx_leng[np.where(mask, ved, 0)] * mask
    ll = grid.ed_leng[np.where(mask, ved, 0)] * mask
    mean_d = d.sum(axis=1) / n
    mean_l = ll.sum(axis=1) / n
    Tt = _tangent(T, P[:, None, :])
    r = np.sqrt(np.sum(Tt * Tt, axis=2)) * mask
    mean_r = r.sum(axis=1) / n
    xs, cells, slots = [], [], []
    for j in range(6):
        c = np.nonzero(j < n)[0]
        nc = n[c]
        f = np.zeros((c.size, NFEAT))
        for q, dj in enumerate((0, -1, 1, -2, 2, 3)):
            f[:, q] = 10.0 * (R[c, (j + dj) % nc] - 1.0 / nc)
        f[:, 6] = (nc == 5).astype(np.float64)
        D = Tt[c, j]
        D = D / np.sqrt(np.sum(D * D, axis=1))[:, None]
        Q = np.cross(P[c], D)
        f[:, 7] = 10.0 * np.sum(O[c] * D, axis=1) / sA[c]
        f[:, 8] = 10.0 * np.sum(O[c] * Q, axis=1) / sA[c]
        e0 = ved[c, j]
        e1 = ved[c, (j + 1) % nc]
        f[:, 9] = 10.0 * (grid.edhx_leng[e0] / mean_d[c] - 1.0)
        f[:, 10] = 10.0 * (grid.edhx_leng[e1] / mean_d[c] - 1.0)
        f[:, 11] = 10.0 * (grid.ed_leng[e0] / mean_l[c] - 1.0)
        f[:, 12] = 10.0 * (grid.ed_leng[e1] / mean_l[c] - 1.0)
        f[:, 13] = 10.0 * (r[c, j] / mean_r[c] - 1.0)
        xs.append(f)
        cells.append(c)
        slots.append(np.full(c.size, j))
    return (np.concatenate(xs).astype(np.float32), np.concatenate(cells),
            np.concatenate(slots))


def trsk_weights(nnb, R):
    """calc_trisk_weights (interpack.f90:4046-4095) from kite fractions
    R[nv, 6]: w[c][j][i] = trskw_c(i, j) = sum_{k=i}^{j-1} R_c(k) - 1/2
    (cyclic, summed in the reference's order), 0 on the diagonal."""
    nv = R.shape[0]
    w = np.zeros((nv, 6, 6))
    for nn in (5, 6):
        c = np.nonzero(nnb == nn)[0]
        Rc = R[c]
        for i in range(nn):
            for j in range(nn):
                if i == j:
                    continue
                s = np.zeros(c.size)
                if j < i:
                    for k in range(i, nn):
                        s = s + Rc[:, k]
                    for k in range(0, j):
                        s = s + Rc[:, k]
                else:
                    for k in range(i, j):
                        s = s + Rc[:, k]
                w[c, j, i] = s - 0.5
    return w


def apply_outputs(grid: Grid, y, cell, slot):
    """(R', trskw') from network outputs y for (cell, slot): dR = OUT_SCALE y,
    projected to sum zero over each cell's slots."""
    nv = grid.nv
    n = grid.nnb.astype(np.int64)
    dR = np.zeros((nv, 6))
    dR[cell, slot] = OUT_SCALE * np.asarray(y, dtype=np.float64)
    mask = np.arange(6)[None, :] < n[:, None]
    dR = (dR - (dR.sum(axis=1) / n)[:, None]) * mask
    R = grid.hx_hxtr_area.reshape(nv, 6) + dR
    return R, trsk_weights(n, R)


def with_weights(grid: Grid, R, w) -> Grid:
    """A shallow copy of grid whose kite fractions and TRSK weights are R and
    w (the mesh the learned handle steps, for the oracle and the tests)."""
    import copy
    g2 = copy.copy(grid)
    g2._struct = None
    g2.hx_hxtr_area = np.ascontiguousarray(np.asarray(R).reshape(grid.hx_hxtr_area.shape))
    g2.hx_trskw = np.ascontiguousarray(np.asarray(w).reshape(grid.hx_trskw.shape))
    return g2


def corrected_grid(grid: Grid, mlp, return_outputs: bool = False):
    """The grid with the network's kite-fraction corrections applied."""
    x, cell, slot = kite_inputs(grid)
    y = mlp.forward(learned.to_bf16_bits(x)).astype(np.float64)
    R, w = apply_outputs(grid, y, cell, slot)
    g2 = with_weights(grid, R, w)
    return (g2, y) if return_outputs else g2


# ---- least-squares targets ------------------------------------------------
def _design(grid: Grid, u):
    """Sparse matrix [ne, 6 nv] of the change of TRSK's tangential velocity
    at each edge with respect to z_c(m), where dR_c = z_c - mean(z_c)."""
    nv = grid.nv
    n = grid.nnb.astype(np.int64)
    ved = grid.v_ed.astype(np.int64) - 1
    ttg = grid.hx_ttgout.reshape(nv, 6).astype(np.float64)
    tnr = grid.hx_tnrccw.reshape(nv, 6).astype(np.float64)
    rows, cols, vals = [], [], []
    for nn in (5, 6):
        c = np.nonzero(n == nn)[0]
        for i in range(nn):
            e = ved[c, i]
            for j in range(nn):
                if i == j:
                    continue
                k = ved[c, j]
                coef = -(u[k] * grid.edhx_leng[k] * ttg[c, j] * tnr[c, i]) / grid.ed_leng[e]
                length = (j - i) % nn
                for m in range(nn):
                    inr = 1.0 if (m - i) % nn < length else 0.0
                    rows.append(e)
                    cols.append(6 * c + m)
                    vals.append(coef * (inr - length / nn))
    A = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(grid.ne, 6 * nv))
    return A.tocsr()


def lsq_targets(grid: Grid, seeds, lmax: int, damp: float = 1e-3, iters: int = 3000):
    """Kite-fraction corrections dR[nv, 6] (sum zero per cell) that minimise
    TRSK's tangential reconstruction error over seeded smooth fields (ridge
    least squares, LSQR)."""
    st = learned.stencil(grid)
    blocks, rhs = [], []
    for s in seeds:
        u, ut = learned.velocity_sample(grid, lmax=lmax, seed=s)
        blocks.append(_design(grid, u))
        rhs.append(ut - learned.trsk_tangent_np(grid, u, st))
    A = sp.vstack(blocks).tocsr()
    z = sla.lsqr(A, np.concatenate(rhs), damp=damp, atol=1e-12, btol=1e-12, iter_lim=iters)[0]
    z = z.reshape(grid.nv, 6)
    n = grid.nnb.astype(np.int64)
    mask = np.arange(6)[None, :] < n[:, None]
    z = z * mask
    return (z - (z.sum(axis=1) / n)[:, None]) * mask


def reconstruction_error(grid: Grid, u, ut):
    """Relative RMS error of TRSK's tangential velocity on this grid's
    weights."""
    t = learned.trsk_tangent_np(grid, u, learned.stencil(grid))
    return float(np.sqrt(np.mean((t - ut) ** 2) / np.mean(ut ** 2)))
