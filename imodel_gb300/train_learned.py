"""Trains the learned TRSK correction on the GPU and saves its parameters.

Training set (as the benchmark configuration describes): seeded smooth
velocity fields -- spherical harmonics of degree <= 48 with an l^-2
coefficient spectrum, rotational plus divergent parts -- on icosahedral
level 7 (491,520 edges per field); inputs and targets from
imodel_gb300.learned; Adam (lr 1e-3) on batches of 65,536 edges, run by the
library's tensor-core kernels (include/imodel_mlp.h).  The fields are
sampled by a pool of worker processes started with "spawn" before any GPU
work.

    python -m imodel_gb300.train_learned --level 7 --fields 256 --steps 4000 \
        --out imodel_gb300/data/trsk_mlp_l7.npy
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import time

import numpy as np


def _sample(args):
    level, seed, lmax = args
    from imodel_gb300 import learned
    from imodel_gb300.mesh import meshbuild
    g = _grid_cache.get(level)
    if g is None:
        g = meshbuild(level, nthreads=1)
        _grid_cache[level] = g
    return learned.training_set(g, [seed], lmax=lmax)


_grid_cache: dict = {}


def build_training_set(level: int, seeds, lmax: int = 48, workers: int = 0):
    workers = workers or max(1, (os.cpu_count() or 1))
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        parts = pool.map(_sample, [(level, s, lmax) for s in seeds])
    return tuple(np.concatenate([p[k] for p in parts]) for k in range(3))


def evaluate(net, levels, lmax, seeds=(10**6 + 1, 10**6 + 2)):
    """Relative L2 error of the tangential velocity, plain TRSK and corrected,
    on fields the network has not seen, on each grid level."""
    from imodel_gb300 import learned
    from imodel_gb300.mesh import meshbuild
    out = []
    for level in levels:
        g = meshbuild(level)
        st = learned.stencil(g)
        for seed in seeds:
            u, ut = learned.velocity_sample(g, lmax=lmax, seed=seed)
            plain = learned.trsk_tangent_np(g, u, st)
            corr = learned.corrected_tangent(g, net, u, st)
            e0 = float(np.sqrt(np.mean((plain - ut) ** 2) / np.mean(ut ** 2)))
            e1 = float(np.sqrt(np.mean((corr - ut) ** 2) / np.mean(ut ** 2)))
            out.append({"level": level, "seed": seed, "trsk": e0, "learned": e1,
                        "gain": e0 / e1})
            print(f"level {level} field {seed}: TRSK {e0:.3e} learned {e1:.3e} "
                  f"gain {e0 / e1:.2f}", flush=True)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--level", type=int, default=7)
    ap.add_argument("--fields", type=int, default=256)
    ap.add_argument("--lmax", type=int, default=48)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--workers", type=int, default=0)
    ap.add_argument("--out", default="")
    a = ap.parse_args(argv)
    t0 = time.time()
    x, t, w = build_training_set(a.level, range(a.seed * 100000, a.seed * 100000 + a.fields),
                              lmax=a.lmax, workers=a.workers)
    t1 = time.time()
    print(f"training set: {x.shape[0]} edges from {a.fields} fields in {t1 - t0:.1f} s")
    from imodel_gb300 import learned
    net = learned.Mlp(params=learned.init_params(a.seed))
    net.load_dataset(x, t, w)
    losses = net.train(a.steps, batch=a.batch, lr=a.lr, seed=a.seed + 1)
    t2 = time.time()
    print(f"trained {a.steps} Adam steps in {t2 - t1:.1f} s: loss {losses[:10].mean():.4f} -> "
          f"{losses[-10:].mean():.4f} (weighted target variance {np.mean(w * t * t):.4f})")
    p = net.get_params()
    report = {"edges": int(x.shape[0]), "fields": a.fields, "level": a.level, "lmax": a.lmax,
              "steps": a.steps, "batch": a.batch, "lr": a.lr, "train_s": t2 - t1,
              "loss_first": float(losses[:10].mean()), "loss_last": float(losses[-10:].mean()),
              "eval": evaluate(net, [a.level, a.level + 1], a.lmax)}
    print(json.dumps(report))
    if a.out:
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        np.save(a.out, p)
        print(f"saved {a.out}")
    return p, losses


if __name__ == "__main__":
    main()
