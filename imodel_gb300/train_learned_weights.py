"""Trains the network of the learned TRSK weights (imodel_gb300/learned_weights.py).

  python -m imodel_gb300.train_learned_weights [--levels 5,6] [--fields 12]
      [--steps 4000] [--batch 65536] [--lr 1e-3] [--out PATH]

1. On each training level, seeded smooth velocity fields (spherical
   harmonics up to degree 12 * 2^(level - 5), rotational and divergent
   parts; their tangential component is exact) give, by ridge least squares,
   the kite-fraction corrections that minimise TRSK's tangential
   reconstruction error there (CPU, sparse LSQR).
2. The network (24 -> 64 -> 64 -> 1, BF16 weights) learns those corrections
   (divided by learned_weights.OUT_SCALE) from the geometry features of each
   kite slot, trained on the GPU by the library's own tensor-core forward,
   backward and Adam kernels (imodel_mlp_train).
3. The parameters are written to --out (default
   imodel_gb300/data/trsk_kite_mlp.npy).

--save-dataset / --load-dataset keep step 1's result in an .npz file.
"""
from __future__ import annotations

import argparse
import os
import time

import numpy as np


def build_dataset(levels, fields, damp=1e-3):
    from .mesh import meshbuild
    from . import learned_weights as lw
    xs, ts = [], []
    for L in levels:
        g = meshbuild(L)
        lmax = 12 * 2 ** (L - 5)
        t0 = time.perf_counter()
        dR = lw.lsq_targets(g, range(fields), lmax, damp=damp)
        x, cell, slot = lw.kite_inputs(g)
        xs.append(x)
        ts.append((dR[cell, slot] / lw.OUT_SCALE).astype(np.float32))
        print(f"level {L}: {x.shape[0]} kite slots, {fields} fields of degree <= {lmax}, "
              f"least squares {time.perf_counter() - t0:.0f} s, target rms {ts[-1].std():.3f}",
              flush=True)
    return np.concatenate(xs), np.concatenate(ts)


def main(argv=None):
    from . import learned, learned_weights as lw
    ap = argparse.ArgumentParser()
    ap.add_argument("--levels", default="5,6")
    ap.add_argument("--fields", type=int, default=12)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=lw.TRAINED_PATH)
    ap.add_argument("--save-dataset", default="")
    ap.add_argument("--load-dataset", default="")
    args = ap.parse_args(argv)
    if args.load_dataset:
        z = np.load(args.load_dataset)
        x, t = z["x"], z["t"]
    else:
        x, t = build_dataset([int(v) for v in args.levels.split(",")], args.fields)
        if args.save_dataset:
            np.savez(args.save_dataset, x=x, t=t)
    net = learned.Mlp(params=learned.init_params(args.seed))
    net.load_dataset(learned.to_bf16_bits(x), t)
    t0 = time.perf_counter()
    losses = net.train(args.steps, batch=args.batch, lr=args.lr, seed=args.seed + 1)
    el = time.perf_counter() - t0
    p = net.get_params()
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    np.save(args.out, p)
    var = float(np.mean(t.astype(np.float64) ** 2))
    print(f"trained {args.steps} Adam steps of batch {args.batch} in {el:.1f} s on the GPU; "
          f"loss {losses[:50].mean():.4f} -> {losses[-50:].mean():.4f} "
          f"(target mean square {var:.4f}); parameters in {args.out}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
