"""Accuracy and throughput runs of the shallow-water configurations.

    python -m imodel_gb300.experiments <run> [--out result.json] [options]

Runs (all on one GPU, seeded synthetic states from imodel_gb300.fields):

  tc2        Williamson case 2 on icos level 5, dt 450 s, 5 days: FP64 and
             FP32 error tables against the steady state (the reference's
             swm_tests numbers).
  balanced   icos level 8, dt 110 s, 10 days, balanced state (degree
             1..64, l^-2 coefficients, max wind 40 m/s): FP32 and FP32 +
             learned correction against the FP64 run of the same grid.
  ensemble   64 members on level 6 (dt 225 s, seeds 0..63) and 16 on
             level 7 (dt 110 s, seeds 100..115), degree <= 32, 5 days, in one
             persistent launch; spot members checked against single runs.
  mountains  level 8, dt 108 s, 10 days, balanced flow over 4 Gaussian
             mountains: plain FP32 and FP32 + learned correction, each
             against an FP64 run on level 9 (dt 54 s) restricted to the
             level-8 cells.
  fixed      level 9 (dt 54 s) FP64, FP32 and FP32 + learned, 10 days,
             each against an FP64 run on level 10 (dt 27 s): h error and
             cell-steps/s at equal error.
  large      level 10, dt 28 s, 2 days, balanced state with an l^-3 energy
             spectrum to degree 256 and max wind 60 m/s: FP32 + learned
             against FP64.

h of a coarser grid is compared with a finer grid's solution by index
restriction: the icosahedral refinement keeps every node of level L as the
first nv(L) nodes of level L+1.  Errors are area-weighted relative L2 and
relative max norms, as error_calc (src/swm.f90:3492-3543).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import time

import numpy as np

DAY = 86400.0


def _pool(workers: int = 0):
    # started before any GPU work
    return mp.get_context("spawn").Pool(workers or max(1, os.cpu_count() or 1))


def rel_errors(x, ref, w):
    d = x - ref
    l2 = float(np.sqrt(np.sum(w * d * d) / np.sum(w * ref * ref)))
    linf = float(np.max(np.abs(d)) / np.max(np.abs(ref)))
    return {"l2": l2, "linf": linf}


def _edge_w(g):
    return g.ed_leng * g.edhx_leng / 2.0


def run(grid, path, h, u, dt, nsteps, bt=None, params=None, chunk=0, testcase=2, wparams=None):
    """One run on the GPU; returns the final state, timing and diagnostics.
    path: "fp64", "fp32", "fp32l" (FP32 + the per-step learned correction,
    parameters `params`), "fp32w" / "fp64w" (the learned TRSK weights,
    parameters `wparams`)."""
    from . import swm
    if path in ("fp32w", "fp64w") and wparams is None:
        from . import learned_weights
        wparams = learned_weights.trained_params()
        if wparams is None:
            raise SystemExit("no trained weights network: run imodel_gb300.train_learned_weights")
    m = swm.SWM(grid, precision="fp64" if path.startswith("fp64") else "fp32", bt=bt,
                learned_params=params if path == "fp32l" else None,
                learned_weights=wparams if path in ("fp32w", "fp64w") else None,
                testcase=testcase)
    try:
        m.set_state(h, u)
        if not path.startswith("fp64"):
            m.autotune(dt, 3)
            m.set_state(h, u)
        d0 = m.diagnostics()
        # the learned path reports when its drift guard switched it off
        guarded = path in ("fp32l", "fp32w")
        chunk = chunk or (256 if guarded else nsteps)
        t0 = time.perf_counter()
        done, off_at = 0, None
        while done < nsteps:
            k = min(chunk, nsteps - done)
            m.advance(dt, k)
            done += k
            if guarded and off_at is None and not m.diagnostics()["learned_active"]:
                off_at = done
        el = time.perf_counter() - t0
        d1 = m.diagnostics()
        hf, uf = m.get_state()
    finally:
        m.close()
    rel = lambda k: (d1[k] - d0[k]) / abs(d0[k]) if d0[k] else d1[k] - d0[k]  # noqa: E731
    return {"h": hf, "u": uf, "seconds": el, "steps": nsteps,
            "cell_steps_per_s": grid.nv * nsteps / el,
            "mass_change": rel("mass"), "tenergy_change": rel("tenergy"),
            "learned_active": bool(d1["learned_active"]), "nan": bool(d1["nan_found"]),
            "learned_off_by_step": off_at}


def _summary(r, keep=("seconds", "steps", "cell_steps_per_s", "mass_change", "tenergy_change",
                      "learned_active", "learned_off_by_step")):
    return {k: r[k] for k in keep}


def _params(args):
    from . import learned
    p = learned.trained_params()
    if p is None:
        raise SystemExit("no trained network: run imodel_gb300.train_learned first")
    return p


def exp_tc2(args, pool):
    from . import swm
    from .mesh import meshbuild
    g = meshbuild(5)
    out = {}
    for prec in ("fp64", "fp32"):
        out[prec] = swm.swm_tests(g, 450.0, 5.0, precision=prec)
    return out


def exp_balanced(args, pool):
    from . import fields, swm
    from .mesh import meshbuild
    g = meshbuild(args.level or 8)
    dt = args.dt or 110.0
    n = swm.ntime_for(args.days or 10.0, dt)
    h, u = fields.balanced_state(g, lmax=64, seed=0, evaluator=fields.PoolEvaluator(pool))
    r64 = run(g, "fp64", h, u, dt, n)
    out = {"level": g.level, "dt": dt, "steps": n, "fp64": _summary(r64)}
    for path in ("fp32", "fp32w", "fp32l"):
        r = run(g, path, h, u, dt, n, params=_params(args) if path == "fp32l" else None)
        out[path] = dict(_summary(r), h_vs_fp64=rel_errors(r["h"], r64["h"], g.hx_areag),
                         u_vs_fp64=rel_errors(r["u"], r64["u"], _edge_w(g)))
    return out


def _member_state(args):
    level, seed = args
    from . import fields
    from .mesh import meshbuild
    g = meshbuild(level, nthreads=1)
    return fields.balanced_state(g, lmax=32, seed=seed)


def exp_ensemble(args, pool):
    from . import swm
    from .mesh import meshbuild
    levels, seeds = (6, 7), (list(range(64)), list(range(100, 116)))
    dts = [225.0, 110.0]
    days = args.days or 5.0
    steps = [swm.ntime_for(days, dt) for dt in dts]
    grids = [meshbuild(l) for l in levels]
    states = [pool.map(_member_state, [(l, s) for s in ss]) for l, ss in zip(levels, seeds)]
    ens = swm.Ensemble(grids, [len(s) for s in seeds])
    try:
        for k in range(2):
            for j, (h, u) in enumerate(states[k]):
                ens.set_state(k, j, h, u)
        tune = ens.tune(dts, 3)
        for k in range(2):
            for j, (h, u) in enumerate(states[k]):
                ens.set_state(k, j, h, u)
        t0 = time.perf_counter()
        ens.advance(dts, steps)
        el = time.perf_counter() - t0
        finals = {(k, j): ens.get_state(k, j) for k, j in ((0, 0), (0, 63), (1, 0), (1, 15))}
    finally:
        ens.close()
    cells = sum(len(s) * g.nv * n for s, g, n in zip(seeds, grids, steps))
    out = {"members": [len(s) for s in seeds], "levels": list(levels), "dt": dts,
           "steps": steps, "seconds": el, "cell_steps_per_s": cells / el, "tuning": tune}
    # spot members: single-instance FP32 and FP64 runs of the same states
    single = [0.0, 0.0]
    checks = []
    for (k, j), (hf, uf) in finals.items():
        g = grids[k]
        h, u = states[k][j]
        r32 = run(g, "fp32", h, u, dts[k], steps[k])
        r64 = run(g, "fp64", h, u, dts[k], steps[k])
        single[k] += r32["seconds"]
        checks.append({"level": levels[k], "member": j,
                       "h_vs_single_fp32": rel_errors(hf, r32["h"], g.hx_areag),
                       "h_vs_fp64": rel_errors(hf, r64["h"], g.hx_areag),
                       "u_vs_fp64": rel_errors(uf, r64["u"], _edge_w(g))})
    out["checks"] = checks
    # the same work as separate graph-launched single runs, from the spot
    # members' timings (two per level)
    out["separate_runs_estimate_s"] = (single[0] / 2.0) * len(seeds[0]) + \
        (single[1] / 2.0) * len(seeds[1])
    return out


def _restrict_errors(r, ref, g):
    return rel_errors(r["h"], ref["h"][: g.nv], g.hx_areag)


def exp_mountains(args, pool):
    from . import fields, swm
    from .mesh import meshbuild
    days = args.days or 10.0
    gc, gf = meshbuild(8), meshbuild(9)
    dtc, dtf = 108.0, 54.0
    nc, nf = swm.ntime_for(days, dtc), swm.ntime_for(days, dtf)
    ev = fields.PoolEvaluator(pool)
    btc, btf = fields.gaussian_mountains(gc, seed=0), fields.gaussian_mountains(gf, seed=0)
    hc, uc = fields.balanced_state(gc, lmax=64, seed=0, bt=btc, evaluator=ev)
    hf, uf = fields.balanced_state(gf, lmax=64, seed=0, bt=btf, evaluator=ev)
    ref = run(gf, "fp64", hf, uf, dtf, nf, bt=btf)
    out = {"coarse": {"level": 8, "dt": dtc, "steps": nc},
           "reference": dict(_summary(ref), level=9, dt=dtf, path="fp64")}
    p = _params(args)
    for path in ("fp64", "fp32", "fp32w", "fp32l"):
        r = run(gc, path, hc, uc, dtc, nc, bt=btc, params=p)
        # the topography is the same at the shared nodes: depth error =
        # free-surface error
        out[path] = dict(_summary(r), h_vs_l9_fp64=_restrict_errors(r, ref, gc))
    return out


def exp_fixed(args, pool):
    from . import fields, swm
    from .mesh import meshbuild
    days = args.days or 10.0
    lc = args.level or 9
    gc, gf = meshbuild(lc), meshbuild(lc + 1)
    dtc = args.dt or 54.0
    dtf = dtc / 2.0
    nc, nf = swm.ntime_for(days, dtc), swm.ntime_for(days, dtf)
    ev = fields.PoolEvaluator(pool)
    hc, uc = fields.balanced_state(gc, lmax=64, seed=0, evaluator=ev)
    if args.load_ref:
        # the fine run's h at the coarse nodes, saved by an earlier --save-ref
        d = np.load(args.load_ref)
        ref = {"h": d["h"]}
        out = {"coarse": {"level": lc, "dt": dtc, "steps": nc},
               "reference": {k: d[k].item() for k in d.files if k != "h"}}
    else:
        hf, uf = fields.balanced_state(gf, lmax=64, seed=0, evaluator=ev)
        r = run(gf, args.ref_precision, hf, uf, dtf, nf, chunk=2000)
        ref = {"h": r["h"][: gc.nv]}
        out = {"coarse": {"level": lc, "dt": dtc, "steps": nc},
               "reference": dict(_summary(r), level=lc + 1, dt=dtf, path=args.ref_precision)}
        if args.save_ref:
            np.savez(args.save_ref, h=ref["h"],
                     **{k: np.array(v) for k, v in out["reference"].items() if v is not None})
    paths = [q for q in args.paths.split(",") if q]
    p = _params(args) if "fp32l" in paths else None
    for path in paths:
        r = run(gc, path, hc, uc, dtc, nc, params=p)
        out[path] = dict(_summary(r), h_vs_ref=_restrict_errors(r, ref, gc))
    for q in ("fp32l", "fp32w"):
        if q in out and "fp64" in out:
            out[f"speedup_{q}_vs_fp64"] = (out[q]["cell_steps_per_s"] /
                                           out["fp64"]["cell_steps_per_s"])
    return out


def exp_large(args, pool):
    from . import fields, swm
    from .mesh import meshbuild
    g = meshbuild(10)
    dt = 28.0
    n = swm.ntime_for(args.days or 2.0, dt)
    h, u = fields.balanced_state(g, lmax=256, seed=0, exponent=-3.0, umax=60.0,
                                 evaluator=fields.PoolEvaluator(pool))
    r64 = run(g, "fp64", h, u, dt, n, chunk=2000)
    out = {"level": 10, "dt": dt, "steps": n, "fp64": _summary(r64)}
    for path in ("fp32", "fp32w", "fp32l"):
        r = run(g, path, h, u, dt, n, params=_params(args) if path == "fp32l" else None)
        out[path] = dict(_summary(r), h_vs_fp64=rel_errors(r["h"], r64["h"], g.hx_areag),
                         u_vs_fp64=rel_errors(r["u"], r64["u"], _edge_w(g)))
    return out


def exp_williamson(args, pool):
    """Cases 1, 5, 6 and 21 of the reference (imodel_gb300/testcases.py) at
    one level (default 7), time steps scaled from level 5 (900, 300, 225 and
    225 s) by the grid spacing.  Case 1 (cosine bell, one 12-day rotation)
    against its initial state, the exact solution; cases 5 (15 days), 6 (14
    days) and 21 (Galewsky jet, 6 days) FP32 and FP32 + learned against
    FP64, with mass and energy changes."""
    from . import swm, testcases
    from .mesh import meshbuild
    lvl = args.level or 7
    g = meshbuild(lvl)
    scale = 2.0 ** (5 - lvl)
    out = {"level": lvl}
    for case, dt5, days in ((1, 900.0, 12.0), (5, 300.0, 15.0), (6, 225.0, 14.0),
                            (21, 225.0, 6.0)):
        dt = dt5 * scale
        n = swm.ntime_for(days, dt)
        h, u, bt = testcases.initialize_fields(g, case)
        btp = bt if np.any(bt != 0) else None
        res = {"dt": dt, "steps": n, "days": days}
        r64 = run(g, "fp64", h, u, dt, n, bt=btp, testcase=case)
        res["fp64"] = _summary(r64)
        paths = ("fp32",) if case < 2 else ("fp32", "fp32w", "fp32l")
        for path in paths:
            r = run(g, path, h, u, dt, n, bt=btp, testcase=case,
                    params=_params(args) if path == "fp32l" else None)
            res[path] = dict(_summary(r), h_vs_fp64=rel_errors(r["h"], r64["h"], g.hx_areag),
                             u_vs_fp64=rel_errors(r["u"], r64["u"], _edge_w(g)))
            if case == 1:
                res[path]["h_vs_exact"] = rel_errors(r["h"], h, g.hx_areag)
        if case == 1:
            res["fp64"]["h_vs_exact"] = rel_errors(r64["h"], h, g.hx_areag)
        out[f"case{case}"] = res
    return out


def exp_case2(args, pool):
    """Williamson case 2 (a steady flow with a known answer, swm.f90:1205-1326)
    at levels 5 to args.level (default 9) for args.days (default 5), plain
    FP32 TRSK against FP32 with the learned TRSK weights: h and u errors
    against the initial (exact) state.  The network was fitted on levels 5
    and 6 only.  dt = 900 s at level 5, halved per level."""
    from . import swm
    from .mesh import meshbuild
    days = args.days or 5.0
    out = {"days": days}
    for lvl in range(5, (args.level or 9) + 1):
        g = meshbuild(lvl, device=0)
        h, u = swm.initialize_fields_tc2(g)
        dt = 900.0 * 2.0 ** (5 - lvl)
        n = swm.ntime_for(days, dt)
        row = {"dt": dt, "steps": n}
        for path in ("fp32", "fp32w"):
            r = run(g, path, h, u, dt, n)
            row[path] = dict(_summary(r), h_err=rel_errors(r["h"], h, g.hx_areag),
                             u_err=rel_errors(r["u"], u, _edge_w(g)))
        row["h_l2_ratio"] = row["fp32"]["h_err"]["l2"] / row["fp32w"]["h_err"]["l2"]
        row["u_l2_ratio"] = row["fp32"]["u_err"]["l2"] / row["fp32w"]["u_err"]["l2"]
        out[f"level{lvl}"] = row
    return out


def exp_schemes(args, pool):
    """The method wrappers on FP64 and FP32 handles: cell-steps/s over
    args.days (default 0.5) of a seeded balanced state at args.level
    (default 8; dt 110 s scaled by the grid spacing), and the FP32 state's
    relative L2 distance from the FP64 one after the run."""
    from . import fields
    from .mesh import meshbuild
    from .swm import SWM
    lvl = args.level or 8
    g = meshbuild(lvl)
    dt = 110.0 * 2.0 ** (8 - lvl)
    n = swm_steps(args.days or 0.5, dt)
    h, u = fields.balanced_state(g, lmax=32, seed=0, evaluator=fields.PoolEvaluator(pool))
    out = {"level": lvl, "dt": dt, "steps": n}
    for scheme in ("trsk10", "pxt16", "gass18", "dtred"):
        row = {}
        r64 = None
        for prec in ("fp64", "fp32"):
            m = SWM(g, prec, scheme=scheme)
            m.set_state(h, u)
            m.advance(dt, 2)                     # graph capture and warm-up
            m.set_state(h, u)
            t0 = time.perf_counter()
            m.advance(dt, n)
            hh, uu = m.get_state()
            sec = time.perf_counter() - t0
            m.close()
            row[prec] = {"cell_steps_per_s": g.nv * n / sec, "seconds": sec}
            if prec == "fp64":
                r64 = (hh, uu)
            else:
                row[prec]["h_vs_fp64"] = rel_errors(hh, r64[0], g.hx_areag)
                row[prec]["u_vs_fp64"] = rel_errors(uu, r64[1], _edge_w(g))
        row["fp32_over_fp64"] = row["fp32"]["cell_steps_per_s"] / row["fp64"]["cell_steps_per_s"]
        out[scheme] = row
    return out


def exp_apvm(args, pool):
    """APVM (pvspar 0.5) on a seeded balanced state at args.level (default
    9, dt 110 s scaled by the grid spacing): cell-steps/s of the FP64 step
    and of the FP32 step in each variant and as autotuned, over args.days
    (default 0.1) after a 2-step warm-up, with FP32's distance from FP64."""
    from . import fields
    from .mesh import meshbuild
    from .swm import SWM
    lvl = args.level or 9
    g = meshbuild(lvl, device=0)
    dt = 110.0 * 2.0 ** (8 - lvl)
    n = swm_steps(args.days or 0.1, dt)
    h, u = fields.balanced_state(g, lmax=32, seed=0, evaluator=fields.PoolEvaluator(pool))
    out = {"level": lvl, "dt": dt, "steps": n}
    r64 = None
    for name, prec, variant in (("fp64", "fp64", None), ("fp32_v0", "fp32", 0),
                                ("fp32_v1", "fp32", 1), ("fp32_v2", "fp32", 2),
                                ("fp32_tuned", "fp32", -1)):
        m = SWM(g, prec)
        m.set_apvm(0.5, dt)
        m.set_state(h, u)
        row = {}
        if variant == -1:
            row["tuning"] = m.autotune(dt)
        elif variant is not None:
            m.set_tuning(variant=variant)
        m.advance(dt, 2)
        m.set_state(h, u)
        t0 = time.perf_counter()
        m.advance(dt, n)
        hh, uu = m.get_state()
        sec = time.perf_counter() - t0
        m.close()
        row.update({"cell_steps_per_s": g.nv * n / sec, "seconds": sec})
        if r64 is None:
            r64 = (hh, uu)
        else:
            row["h_vs_fp64"] = rel_errors(hh, r64[0], g.hx_areag)
            row["u_vs_fp64"] = rel_errors(uu, r64[1], _edge_w(g))
        out[name] = row
    return out


def exp_moist(args, pool):
    """Throughput of the moist model (FP64 and FP32 GPU handles, test case
    2, trsk and upw1 advection; FP32's relative L2 distance from FP64) against
    the dry FP64 and FP32 steps from the same h and u, at levels 5 to
    args.level (default 9), dt 110 s scaled by the grid spacing; each timed
    over args.days (default 0.1, at least 100 steps) after a 2-step
    warm-up."""
    from .mesh import meshbuild
    from .moist import Moist, moist_fields
    from .swm import SWM
    out = {}
    for lvl in range(5, (args.level or 9) + 1):
        g = meshbuild(lvl, device=0)
        dt = 110.0 * 2.0 ** (8 - lvl)
        n = max(swm_steps(args.days or 0.1, dt), 100)
        f = moist_fields(g, 2)
        row = {"dt": dt, "steps": n, "cells": g.nv}
        ref = {}
        for prec in ("fp64", "fp32"):
            for adv in ("trsk", "upw1"):
                m = Moist(g, 2, f, advection=adv, precision=prec)
                m.set_state(f)
                m.advance(dt, 2)
                m.set_state(f)
                t0 = time.perf_counter()
                m.advance(dt, n)
                sec = time.perf_counter() - t0
                st = m.get_state()
                m.close()
                r = {"cell_steps_per_s": g.nv * n / sec, "seconds": sec}
                if prec == "fp64":
                    ref[adv] = st
                else:
                    r["h_vs_fp64"] = rel_errors(st["h"], ref[adv]["h"], g.hx_areag)
                    r["hqv_vs_fp64"] = rel_errors(st["hqv"], ref[adv]["hqv"], g.hx_areag)
                row[f"moist_{prec}_{adv}"] = r
        for prec in ("fp64", "fp32"):
            m = SWM(g, prec)
            m.set_state(f["h"], f["u"])
            m.advance(dt, 2)
            m.set_state(f["h"], f["u"])
            t0 = time.perf_counter()
            m.advance(dt, n)
            m.get_state()
            sec = time.perf_counter() - t0
            m.close()
            row[f"dry_{prec}"] = {"cell_steps_per_s": g.nv * n / sec, "seconds": sec}
        out[f"level{lvl}"] = row
    return out


def swm_steps(days, dt):
    from . import swm
    return swm.ntime_for(days, dt)


def exp_mesh(args, pool):
    """Grid build times through the C ABI (imodel_mesh_build on all host
    threads against imodel_mesh_build_gpu on device 0), levels 8 to
    args.level (default 10), each the best of two builds."""
    import ctypes

    from . import _capi
    lib = _capi.mesh_lib()
    out = {}
    for lvl in range(8, (args.level or 10) + 1):
        row = {}
        for name, call in (("host", lambda h: lib.imodel_mesh_build(lvl, 0, 0, h)),
                           ("gpu", lambda h: lib.imodel_mesh_build_gpu(lvl, 0, 0, h))):
            best = None
            for _ in range(2):
                h = ctypes.c_void_p()
                t0 = time.perf_counter()
                rc = call(ctypes.byref(h))
                dt = time.perf_counter() - t0
                lib.imodel_mesh_free(h)
                if rc != 0:
                    raise RuntimeError(f"{name} build of level {lvl} failed: {rc}")
                best = dt if best is None else min(best, dt)
            row[f"{name}_s"] = best
        row["cells"] = 10 * 4 ** lvl + 2
        out[f"level{lvl}"] = row
    return out


RUNS = {"tc2": exp_tc2, "mesh": exp_mesh, "moist": exp_moist, "apvm": exp_apvm, "schemes": exp_schemes, "case2": exp_case2, "williamson": exp_williamson, "balanced": exp_balanced, "ensemble": exp_ensemble,
        "mountains": exp_mountains, "fixed": exp_fixed, "large": exp_large}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("runs", nargs="+", choices=sorted(RUNS))
    ap.add_argument("--out", default="")
    ap.add_argument("--days", type=float, default=0.0)
    ap.add_argument("--level", type=int, default=0)
    ap.add_argument("--dt", type=float, default=0.0)
    ap.add_argument("--ref-precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--workers", type=int, default=0)
    ap.add_argument("--paths", default="fp64,fp32,fp32w",
                    help="coarse runs of 'fixed': fp64, fp32, fp32w (FP32 + learned TRSK "
                         "weights), fp64w, fp32l (FP32 + per-step learned correction)")
    ap.add_argument("--save-ref", default="", help="'fixed': save the fine run's h (.npz)")
    ap.add_argument("--load-ref", default="", help="'fixed': reuse a saved fine run")
    a = ap.parse_args(argv)
    pool = _pool(a.workers)
    results = {}
    try:
        for name in a.runs:
            t0 = time.time()
            results[name] = RUNS[name](a, pool)
            results[name]["wall_s"] = time.time() - t0
            print(json.dumps({name: results[name]}), flush=True)
            if a.out:
                with open(a.out, "w") as f:
                    json.dump(results, f, indent=1)
    finally:
        pool.close()
        pool.join()
    return results


if __name__ == "__main__":
    main()
