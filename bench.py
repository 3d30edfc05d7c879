#!/usr/bin/env python
"""Throughput of the GB300 TRSK shallow-water step (cell-steps/s).

Workload: icosahedral level 9 (2,621,442 cells, 7,864,320 edges,
5,242,880 triangles), classic RK4, trsk10 / HTC / geodesic areas, dt = 55 s,
from a seeded balanced state (streamfunction of real spherical harmonics of
degree 1..64 with N(0,1) coefficients times l^-2, seed 0, scaled to a
40 m/s maximum wind; h from linear balance, mean g h = 2.94e4; flat
bottom).  One "step" is one RK4 time step of the whole grid.

  value      cell-steps/s of the FP32 path with the learned TRSK weights
             (a per-kite-slot MLP, evaluated once on the tensor cores when
             the handle is created, corrects the kite fractions TRSK builds
             its weights from), state resident in HBM (graph-replayed
             steps, CUDA events on the library's stream)
  fp32_step_net  the FP32 path with the per-step learned correction (a
             per-edge MLP on the stencil velocities, once per step)
  fp32_plain the same without the learned correction
  fp64       the same for the FP64 reference-order path, with its own
             end-to-end figure
  e2e        cell-steps/s of the headline path through the C ABI call
             imodel_swm_step with pinned host buffers: every step copies h
             and u (FP64) to the device and back inside the timed region
  error_vs_fp64  relative L2 and max-norm differences of the FP32 and
             FP32 + learned states from the FP64 state after the same steps
             from the same start (the learned schemes differ from TRSK by
             design: their accuracy is measured against finer runs)
  roofline   the dominant stencil kernel against the measured HBM copy
             bandwidth; mlp_roofline the per-step network kernel against HBM
             and the measured BF16 tensor throughput; step_roofline the whole step
             with the layout's own bytes per cell-step beside the 2000 B
             model
  cpu_baseline  the CPU oracle (C++ restatement of the Fortran, OpenMP on
             all host threads) on a bounded sample of the same workload
  setup      seconds to build the grid (host threads; geometry on the GPU)
             and to create each path's handle (layout, learned weights)

``--impl reference`` times that CPU implementation alone and prints its line.
Run under torchrun for N GPUs: each rank advances its own replica (no data
exchange), timing is the max over ranks and value sums all ranks' cells.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SWM cell-steps/s at icos-L9, plain FP64 vs FP32+learned at fixed error; HBM GB/s"
UNIT = "cell-steps/s"
LEVEL = 9
DT = 55.0
# the seeded balanced state of the workload
STATE = {"lmax": 64, "seed": 0, "exponent": -2.0, "umax": 40.0, "gh0": 2.94e4}
STATE_NAME = ("seeded balanced state (SH degree 1..64, l^-2, seed 0, max wind 40 m/s, "
              "mean gh 2.94e4)")


def bench_state(g, workers: int = 0):
    """The workload's initial (h, u): the spectral synthesis at every cell
    and edge is split over a spawn process pool (started before any GPU
    work in this process)."""
    import multiprocessing as mp
    from imodel_gb300 import fields
    n = workers or max(1, os.cpu_count() or 1)
    with mp.get_context("spawn").Pool(n) as pool:
        return fields.balanced_state(g, evaluator=fields.PoolEvaluator(pool, chunk=1 << 18),
                                     **STATE)


def rel_errors(x, ref, w):
    """Relative L2 (weighted as error_calc weights cells and edges) and
    max-norm difference of x from ref."""
    d = np.asarray(x, dtype=np.float64) - ref
    return {"l2": float(np.sqrt(np.sum(w * d * d) / np.sum(w * ref * ref))),
            "linf": float(np.max(np.abs(d)) / np.max(np.abs(ref)))}


# ---------------------------------------------------------------------------
# CUDA runtime helpers (events, pinned memory) through ctypes
# ---------------------------------------------------------------------------
class Cudart:
    def __init__(self):
        from imodel_gb300 import _build
        path = os.path.join(_build._cuda_lib_dir(), "libcudart.so")
        self.lib = ctypes.CDLL(path if os.path.exists(path) else "libcudart.so")
        L = self.lib
        L.cudaEventCreate.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
        L.cudaEventRecord.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.cudaEventSynchronize.argtypes = [ctypes.c_void_p]
        L.cudaEventElapsedTime.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_void_p,
                                           ctypes.c_void_p]
        L.cudaEventDestroy.argtypes = [ctypes.c_void_p]
        L.cudaStreamSynchronize.argtypes = [ctypes.c_void_p]
        L.cudaMallocHost.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
        L.cudaFreeHost.argtypes = [ctypes.c_void_p]
        L.cudaSetDevice.argtypes = [ctypes.c_int]

    def event(self):
        e = ctypes.c_void_p()
        assert self.lib.cudaEventCreate(ctypes.byref(e)) == 0
        return e

    def record(self, ev, stream):
        assert self.lib.cudaEventRecord(ev, ctypes.c_void_p(stream)) == 0

    def elapsed_ms(self, a, b):
        assert self.lib.cudaEventSynchronize(b) == 0
        ms = ctypes.c_float()
        assert self.lib.cudaEventElapsedTime(ctypes.byref(ms), a, b) == 0
        return float(ms.value)

    def sync(self):
        self.lib.cudaDeviceSynchronize()

    def pinned(self, n):
        p = ctypes.c_void_p()
        assert self.lib.cudaMallocHost(ctypes.byref(p), n * 8) == 0
        arr = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_double)), shape=(n,))
        return p, arr


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """The ranks of a torchrun launch: one replica per GPU (NCCL); the
    barrier around the timed region and the maximum of the ranks' times.
    backend="gloo" runs the same on CPU tensors (multi-process tests)."""

    def __init__(self, device, backend: str = "nccl"):
        self.ws, self.rank, self.local = dist_env()
        self.torch = None
        self.dev = "cuda" if backend == "nccl" else "cpu"
        if self.ws > 1:
            import torch
            import torch.distributed as dist
            if backend == "nccl":
                torch.cuda.set_device(device)
            dist.init_process_group(backend)
            self.torch, self.dist = torch, dist

    def barrier(self):
        if self.torch is not None:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.torch is None:
            return x
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.torch is not None:
            self.dist.destroy_process_group()


def kernel_bytes(nv, ne, nt, precision, variant=0):
    """Algorithmic bytes of one launch of each stage kernel: every array
    element the kernel reads or writes counted once (gathered arrays count
    once per element, not once per gather)."""
    w = 4 if precision == "fp32" else 8
    # triangle: f, 3 circulation coefs, 3 edge idx, 3 kite coefs, 3 cell idx,
    # q out; gathers u and h
    tri = nt * (w + 3 * w + 3 * 4 + 3 * w + 3 * 4 + w) + ne * w + nv * w
    if precision == "fp32" and variant in (1, 2):
        if variant == 2:
            # the triangle record: 40 bytes (6 16-bit indices, f in the
            # record), 8 bytes of bases per warp of 32 triangles
            tri = nt * (40 + 8 / 32 + w) + ne * w + nv * w
        # cell: meta, 1/(A a), b, 6 slots x (edge, neighbour, triangle idx,
        # kite fraction, KE weight, ttgout*d); h, y_n, acc r/w, y_out, B out,
        # 6 PV-flux contributions out; gathers u and q
        cell = nv * (4 + 4 + 4 + 6 * 24 + 4 + 4 + 8 + 4 + 4 + 6 * 4) + ne * w + nt * w
        # edge: 2 cell words, 1/(l a), y_n, acc r/w, y_out; gathers B and
        # the cells' PV-flux contributions
        edge = ne * (8 + 4 + 4 + 8 + 4) + nv * 4 + nv * 6 * 4
        return {"triangle": tri, "edge_pre": 0, "cell": cell, "edge": edge}
    edge_pre = ne * (8 + 8 + w + 3 * w) + nv * w + nt * w
    cell = nv * (1 + 6 * 4 + 6 * w + 6 * w + w + w + w + 2 * w + w + w) + 2 * ne * w
    edge = ne * (8 + w + w + 1 + 10 * 4 + 10 * w + w + 2 * w + w) + nv * w + ne * w
    if precision == "fp64":
        # FP64 path reads d_k (edhx%leng) per stencil edge and 1 extra coef
        edge += ne * w
        cell += ne * w
    return {"triangle": tri, "edge_pre": edge_pre, "cell": cell, "edge": edge}


def kernel_names(variant):
    if variant == 2:
        return {"triangle": "k_tri32c", "edge_pre": "", "cell": "k_cell32v2",
                "edge": "k_edge32v2"}
    v2 = "v2" if variant == 1 else ""
    return {"triangle": "k_tri32", "edge_pre": "k_edge_pre32", "cell": "k_cell32" + v2,
            "edge": "k_edge32" + v2}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def cpu_baseline_sample(grid, h, u, budget_s=15.0, nthreads=0):
    """Times the CPU oracle on whole RK4 steps of the same grid and state
    until about budget_s seconds have passed."""
    import oracle
    nthreads = nthreads or (os.cpu_count() or 1)
    o = oracle.Oracle(grid, 2, nthreads=nthreads)
    o.ode_rk4(h, u, DT)  # warm-up step (page-in, thread pool)
    steps, t0 = 0, time.perf_counter()
    hh, uu = h, u
    while True:
        hh, uu = o.ode_rk4(hh, uu, DT)
        steps += 1
        el = time.perf_counter() - t0
        if el >= budget_s or steps >= 1000:
            break
    return {"value": grid.nv * steps / el, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{steps} RK4 steps of icos-L{grid.level} ({grid.nv} cells) from the "
                      f"workload's state in {el:.1f} s, C++ oracle, OpenMP {nthreads} threads"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from imodel_gb300 import _build
    from imodel_gb300.mesh import meshbuild
    import oracle
    _build.build_mesh_lib()
    oracle.build()
    g = meshbuild(args.level)
    h, u = bench_state(g)
    nth = os.cpu_count() or 1
    o = oracle.Oracle(g, 2, nthreads=nth)
    hh, uu = h, u
    for _ in range(max(args.warmup, 1)):
        hh, uu = o.ode_rk4(hh, uu, DT)
    budget = 150.0
    steps, t0 = 0, time.perf_counter()
    while steps < args.steps:
        hh, uu = o.ode_rk4(hh, uu, DT)
        steps += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    value = g.nv * steps / el
    sample = (f"{steps} of {args.steps} requested RK4 steps of icos-L{args.level} "
              f"({g.nv} cells), C++ oracle (restatement of the Fortran), {nth} threads")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * el / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic: " + STATE_NAME,
            "config": config_dict(g, "fp64"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def config_dict(g, path, weights=None):
    learned = "off"
    if path == "fp32l":
        learned = ("learned TRSK weights: per-kite-slot MLP 24-64-64-1 (BF16, tcgen05) "
                   "corrects the kite fractions once at create, TRSK weights rebuilt; "
                   "parameters " + (weights or "none"))
    elif path == "fp32n":
        learned = ("per-edge MLP 24-64-64-1, BF16 tcgen05, once per step; parameters " +
                   (weights or "none"))
    return {"workload": f"icos-L{g.level} TRSK shallow-water RK4 step, trsk10/HTC/geo, "
                        f"dt={DT:g} s, {STATE_NAME}",
            "level": g.level, "cells": g.nv, "edges": g.ne, "triangles": g.nt,
            "precision": "fp64" if path == "fp64" else "fp32",
            "learned_correction": learned,
            "l2": "inputs larger than L2 (state + geometry of several GB per step)",
            "parallelism": "replicas"}


MLP_FLOP_PER_EDGE = 2 * (24 * 64 + 64 * 64 + 64)

# DRAM bytes (read + write) per unit of a launch, from one ncu capture of the
# kernel at icos level 8 (128.0 MB for 655,362 cells), scaled to the
# benchmark's level by the number of cells, as the traffic grows with them.
# DRAM bytes per cell of one launch (ncu at icos level 8, an RK stage that
# reads the accumulator)
TRAFFIC_PER_CELL = {"k_cell32v2": 133.779e6 / 655362}


def load_tflops():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


def mlp_bytes(nv, ne, nt):
    """Algorithmic bytes of one launch of the learned-correction kernel: the
    11,264-byte index block of every 128-edge tile, u, q_tr and h gathered
    (each element counted once) and the correction written."""
    tiles = (ne + 127) // 128
    return tiles * 11264 + ne * 4 + nt * 4 + nv * 4 + ne * 4


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--level", type=int, default=LEVEL)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    # switches for profiler runs: time only the listed paths (fp64, fp32 =
    # plain FP32, fp32l = FP32 + learned correction), skip the end-to-end
    # and per-kernel passes
    ap.add_argument("--precisions", default="fp64,fp32,fp32l,fp32n")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-kprof", action="store_true")
    ap.add_argument("--tuning", default="",
                    help="FP32 launch choice 'variant,bs_tri,bs_pre,bs_cell,bs_edge"
                         "[,mlp_gather]' instead of autotuning")
    ap.add_argument("--apvm", type=float, default=0.0,
                    help="pv_stab = apvm with this pvspar on the fp64 and fp32 paths "
                         "(FP32 then runs stencil variant 0)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    ws, rank, local = dist_env()
    from imodel_gb300 import _build, learned, swm
    from imodel_gb300.mesh import meshbuild
    _build.build_all()
    t_set = time.perf_counter()
    g = meshbuild(args.level)
    setup = {"level": args.level, "mesh_host_s": time.perf_counter() - t_set}
    # the state is computed by a process pool before this process touches
    # the GPU
    h, u = bench_state(g, max(1, (os.cpu_count() or 1) // max(ws, 1)))
    cr = Cudart()
    assert cr.lib.cudaSetDevice(local) == 0
    D = Dist(local)
    # the same grid with its geometry built on the GPU (timed only)
    t_set = time.perf_counter()
    meshbuild(args.level, device=local)
    setup["mesh_gpu_s"] = time.perf_counter() - t_set
    setup["create_s"] = {}

    from imodel_gb300 import learned_weights
    params_n = learned.trained_params()
    weights_n = "trained on icos-L7 (imodel_gb300/data/trsk_mlp_l7.npy)"
    if params_n is None:
        params_n = learned.init_params(0)
        weights_n = "untrained (Glorot initial values, seed 0)"
    params_w = learned_weights.trained_params()
    weights_w = "trained on icos-L5 and L6 (imodel_gb300/data/trsk_kite_mlp.npy)"
    if params_w is None:
        params_w = learned.init_params(0)
        weights_w = "untrained (Glorot initial values, seed 0)"
    results = {}
    paths = [p for p in args.precisions.split(",") if p]
    headline = "fp32l" if "fp32l" in paths else "fp32"
    for path in paths:
        t_set = time.perf_counter()
        m = swm.SWM(g, precision="fp64" if path == "fp64" else "fp32", device=local,
                    learned_params=params_n if path == "fp32n" else None,
                    learned_weights=params_w if path == "fp32l" else None)
        setup["create_s"][path] = time.perf_counter() - t_set
        m.set_state(h, u)
        if args.apvm > 0 and path not in ("fp32l", "fp32n"):
            m.set_apvm(args.apvm, DT)
        tuning = None
        if path != "fp64":
            if args.tuning:
                c = [int(x) for x in args.tuning.split(",")]
                m.set_tuning(*c)
                tuning = dict(zip(swm.TUNING_KEYS, c))
            else:
                tuning = m.autotune(DT, 5)
        stream = m.stream()
        m.advance(DT, args.warmup)
        cr.sync()
        ev0, ev1 = cr.event(), cr.event()
        sampler = ClockSampler(local) if path == headline else None
        D.barrier()
        cr.sync()
        if sampler:
            sampler.start()
        cr.record(ev0, stream)
        m.advance(DT, args.steps)
        cr.record(ev1, stream)
        ms = cr.elapsed_ms(ev0, ev1)
        cr.sync()
        clocks = sampler.stop() if sampler else None
        D.barrier()
        ms = D.max(ms)
        diag = m.diagnostics()
        # the state after warmup + steps steps from the common start
        hf, uf = m.get_state()
        prof = None if args.no_kprof else m.profile(DT, 3)
        results[path] = {"ms": ms, "clocks": clocks, "prof": prof, "diag": diag,
                         "tuning": tuning, "launches": m.launch_count(args.steps),
                         "main_kernel": m.main_kernel(), "h": hf, "u": uf}
        if (path == headline or path == "fp64") and not args.no_e2e:
            # e2e through the C ABI with pinned host buffers
            ph, hbuf = cr.pinned(g.nv)
            pu, ubuf = cr.pinned(g.ne)
            hbuf[:] = h
            ubuf[:] = u
            lib = m.lib
            fp = ctypes.POINTER(ctypes.c_double)
            hp, up = ctypes.cast(ph, fp), ctypes.cast(pu, fp)
            for _ in range(2):
                assert lib.imodel_swm_step(m.handle, hp, up, DT, 1) == 0
            D.barrier()
            t0 = time.perf_counter()
            for _ in range(args.e2e_steps):
                rc = lib.imodel_swm_step(m.handle, hp, up, DT, 1)
                assert rc == 0, rc
            el = time.perf_counter() - t0
            D.barrier()
            el = D.max(el)
            results[path]["e2e"] = {"s": el, "steps": args.e2e_steps}
            cr.lib.cudaFreeHost(ph)
            cr.lib.cudaFreeHost(pu)
        m.close()

    full = ("fp64" in results and headline in results and "e2e" in results[headline]
            and results[headline]["prof"])
    if rank == 0 and not full:
        # profiler runs: a short line with the timed paths only
        short = {k: {"ms_per_step": v["ms"] / args.steps} for k, v in results.items()
                 if k in ("fp32", "fp32l", "fp32n", "fp64")}
        print(json.dumps(dict(short, setup=setup)))
    elif rank == 0:
        rh, r64 = results[headline], results["fp64"]
        total_cells = g.nv * ws

        def rate(r):
            return total_cells * args.steps / (r["ms"] / 1000.0)

        def e2e_line(r):
            e = r["e2e"]
            return {"value": total_cells * e["steps"] / e["s"], "unit": UNIT,
                    "h2d_bytes_per_step": 8 * (g.nv + g.ne),
                    "d2h_bytes_per_step": 8 * (g.nv + g.ne),
                    "path": "imodel_swm_step(nsteps=1) with pinned host FP64 h,u"}

        peak, peak_kind = load_peaks()
        variant = rh["tuning"]["variant"]
        kb = kernel_bytes(g.nv, g.ne, g.nt, "fp32", variant)
        prof = {k: v for k, v in rh["prof"].items() if k != "edge_pre" or kb["edge_pre"]}
        dom = max(prof, key=prof.get)
        achieved = kb[dom] / (prof[dom] / 1000.0) / 1e9
        # whole-step bytes: the 2000 B/cell-step model and this layout's own
        # (four stages of the stencil kernels; the learned weights add none)
        layout_step = 4 * sum(kb.values())
        sec_step = rh["ms"] / args.steps / 1000.0
        kernel_ms = dict(prof)
        kname = kernel_names(variant)[dom]
        traffic = TRAFFIC_PER_CELL[kname] * g.nv if kname in TRAFFIC_PER_CELL else None
        wc, we = g.hx_areag, g.ed_leng * g.edhx_leng / 2.0
        err = {}
        for p in ("fp32", "fp32l", "fp32n"):
            if p in results:
                err[p] = {"h": rel_errors(results[p]["h"], r64["h"], wc),
                          "u": rel_errors(results[p]["u"], r64["u"], we)}
        err["steps"] = args.warmup + args.steps
        err["days"] = (args.warmup + args.steps) * DT / 86400.0
        err["reference"] = "the FP64 path's state after the same steps from the same start"
        line = {
            "metric": METRIC, "value": rate(rh), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": rh["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: " + STATE_NAME + " (no dataset)",
            "config": dict(config_dict(g, headline, weights_w if headline == "fp32l" else None),
                           autotuned=rh["tuning"],
                           **({"apvm_pvspar": args.apvm} if args.apvm > 0 else {})),
            "error_vs_fp64": err,
            "fp64": {"value": rate(r64), "unit": UNIT, "ms_per_step": r64["ms"] / args.steps,
                     "kernel_ms": r64["prof"], "dtype": "f64",
                     **({"e2e": e2e_line(r64)} if "e2e" in r64 else {})},
            "kernel_ms": kernel_ms,
            "roofline": {"bound": "hbm", "kernel": kname,
                         "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": peak_kind, "traffic": traffic,
                         "traffic_source": "ncu capture at icos level 8, scaled by cells",
                         "algorithmic_bytes_per_launch": kb[dom]},
            "step_roofline": {
                "bytes_per_cell_step_model": 2000.0,
                "achieved_model": 2000.0 * g.nv / sec_step / 1e9,
                "bytes_per_cell_step_layout": layout_step / g.nv,
                "achieved": layout_step / sec_step / 1e9,
                "peak": peak, "unit": "GB/s", "frac": layout_step / sec_step / 1e9 / peak},
            "e2e": e2e_line(rh),
            "gpu_launches": rh["launches"],
            "clocks": rh["clocks"],
            "setup": setup,
        }
        if "fp32" in results and headline != "fp32":
            line["fp32_plain"] = {"value": rate(results["fp32"]), "unit": UNIT,
                                  "ms_per_step": results["fp32"]["ms"] / args.steps,
                                  "kernel_ms": results["fp32"]["prof"]}
        if headline == "fp32l":
            line["learned_active_after_run"] = bool(rh["diag"]["learned_active"])
        if "fp32n" in results and results["fp32n"]["prof"]:
            # the per-step network: the profile reports it in the edge_pre
            # slot, per stage; it runs once per step
            rn = results["fp32n"]
            nk = dict(rn["prof"])
            mlp_ms = nk.pop("edge_pre") * 4.0
            nk["mlp"] = mlp_ms
            line["fp32_step_net"] = {
                "value": rate(rn), "unit": UNIT, "ms_per_step": rn["ms"] / args.steps,
                "kernel_ms": nk, "learned_active_after_run": bool(rn["diag"]["learned_active"]),
                "config": config_dict(g, "fp32n", weights_n)["learned_correction"]}
            flop = MLP_FLOP_PER_EDGE * g.ne
            tf, tf_kind = load_tflops()
            ach = flop / (mlp_ms / 1000.0) / 1e12
            mb = mlp_bytes(g.nv, g.ne, g.nt)
            line["mlp_roofline"] = {"bound": "hbm", "kernel": "k_mlp_pipe<EdgeTask>",
                                    "achieved": mb / (mlp_ms / 1000.0) / 1e9, "peak": peak,
                                    "unit": "GB/s",
                                    "frac": mb / (mlp_ms / 1000.0) / 1e9 / peak,
                                    "algorithmic_bytes_per_launch": mb,
                                    "tensor": {"achieved": ach, "peak": tf, "unit": "TFLOP/s",
                                               "frac": ach / tf, "peak_source": tf_kind,
                                               "flop_per_launch": flop}}
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_baseline_sample(g, h, u, args.cpu_budget)
        print(json.dumps(line))
    D.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
