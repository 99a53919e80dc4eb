"""Benchmark of the TRANS per-iteration hot path on GB300.

One step = one outer iteration over every interior cell of the workload: one pass of the hot
path for the steady cases (Kchld = 1), Kchld dual-time sub-iterations for the square-cylinder
DES case.  The metric is cell-iterations per second (Mcell-iter/s), each sub-iteration of each
interior cell counting once.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--case cascade|cascade_medium|channel|cylinder]
                  [--precision fp64|mixed] [--impl gb300|reference]

The default line is the FP64 path on the five-block cascade at the benchmark's block sizes
(1,966,080 cells) with sub-objects for the same workload in mixed precision (`mixed`), eight
copies of it in one mixed-precision batch context (`batched`), and a bounded serving stream at
4 requests/s (`serving`, p50/p99 latency).

--impl reference times the reference's algorithm on the host cores: the C++ FP64 restatement
in oracle/ (the Fortran reference cannot be built here), parallel over blocks with OpenMP as
the reference is parallel over blocks with MPI.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from trans_gb300 import abi  # noqa: E402
from trans_gb300 import case as CS  # noqa: E402
from trans_gb300 import cases  # noqa: E402
from trans_gb300.solver import Solver, STATE_FIELDS  # noqa: E402

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0


def init_replicas():
    """One process per GPU (torchrun sets RANK / WORLD_SIZE / LOCAL_RANK): every rank runs an
    independent replica of the workload -- the path does not shard, blocks of one case are
    coupled every sub-iteration -- and the ranks only meet for the barrier and the maximum of
    the timings.  NCCL between GPUs, gloo where no GPU is present."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        if torch.cuda.is_available():
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    return rank, world


def max_over_ranks(x, world):
    """The maximum of x over the ranks (the slowest replica sets the time)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank, seconds, world):
    """Whole-job rate in millions of units per second: every rank processed units_per_rank."""
    return units_per_rank * world / seconds / 1e6


def make_case(name, precision, nk=64, metrics_fn=None):
    """The benchmark workloads: `cascade` is the five-block cascade at the benchmark's block
    sizes (O 257x49x65, H 65x97x65, passage 97x33x65: 1,966,080 cells), `cascade_medium` the
    1,359,872-cell layout of the serving medium level."""
    prec = abi.TRANS_MIXED if precision == "mixed" else abi.TRANS_FP64
    if name == "channel":
        c = cases.channel_bump(precision=prec)
    elif name == "cascade":
        c = cases.cascade(precision=prec, **dict(cases.CASCADE_CONFIG2, nk=nk))
    elif name == "cascade_medium":
        c = cases.cascade(nk=nk, precision=prec)
    elif name == "cylinder":
        c = cases.square_cylinder(precision=prec)
    else:
        raise SystemExit(f"unknown case {name}")
    conns, geo = CS.compute_geometry(c, metrics_fn=metrics_fn)
    st = CS.initial_state(c, geo, Q_dst=c.meta.get("Q_dst", 0.01))
    return c, conns, geo, st


def interior_cells(c):
    return int(sum(np.prod([d - 1 for d in b.dims]) for b in c.blocks))


def sub_iterations(c):
    """Hot-path passes per outer iteration: Kchld dual-time sub-iterations (each counts as a
    cell-iteration), 3 Runge-Kutta stages, or 1."""
    p = c.params
    return 3 if p.IF_RK == 1 else (p.Kchld if p.Kind_Dual != 0 else 1)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        return json.load(open(PEAKS_FILE))
    except Exception:
        return {}


def time_resident(s, ki0, steps):
    ms = C.c_double()
    nb = len(s.blocks)
    norms = (abi.TransNorms * nb)()
    rc = s.lib.trans_time_iterations(s.ctx, ki0, steps, C.byref(ms), norms)
    if rc != 0:
        raise RuntimeError(f"trans_time_iterations failed {rc}: {s.lib.trans_last_error(s.ctx)}")
    return ms.value


# Algorithmic words (FP64 = 8 B) per unit of each kernel class: the compulsory reads and
# writes of one unit (interior cell, or face for the face fluxes) with halos excluded.
ALG_WORDS = {
    "k_face_flux": 51,      # per face: stencil 38 words in, 13 face fluxes out
    "k_resid_tma": 50,      # per face: stencil 38 words in; D of the face's cell, 7 out and 7 in for 2 of 3 directions
    "k_sweep": 24,          # the L -> U hand-off: DeltaQ 7 + Rds 3 + diagonals 2, written and read once
    "k_update": 37, "k_gradient": 46, "k_specrad": 24, "k_lusgs_prep": 60, "k_gather": 46,
}
# FP64 thread-instructions per face of k_face_flux<double> (MDCD + AUSMPW+ + SST), counted by
# ncu (DADD + DMUL + DFMA over the three directions) on the 339,968-cell cascade
# (profiles/k_face_flux_fp64_cascade_339968cells.md), and DRAM bytes per face of the viscous
# and convective kernels the flux is now split into (profiles/launches_cascade_5blk_1966080cells_fp64.md)
FACE_FP64_INST = 2541.0
FACE_DRAM_BYTES = 479.1
FACE_DRAM_SOURCE = ("ncu dram__bytes_read+write per face of the viscous and convective kernels together on the "
                    "491,520-cell cascade, scaled by faces")
# kernel classes that run in FP32 in the mixed path (their algorithmic words are 4 bytes there)
FP32_KERNELS = ("k_face_flux", "k_resid_tma", "k_gather", "k_sweep", "k_gradient")
# bounded serving leg of the default line: 4 requests/s as the serving configuration states,
# for 5 s of arrivals; each request retires at a 0.3 drop of its residual (coarse grids take
# ~580 iterations to it, medium ~690 with the CFL ramp) or after 1,500 iterations, so the leg
# ends within about a minute on one GPU
SERVE_DURATION = 5.0
SERVE_DROP = 0.3
SERVE_MAX_ITERS = 1500


def units(c, kernel):
    """Units a kernel class processes per iteration: faces of all three directions for the
    face fluxes, interior cells otherwise."""
    if kernel in ("k_face_flux", "k_resid_tma"):
        return sum(ni * (nj - 1) * (nk - 1) + (ni - 1) * nj * (nk - 1) + (ni - 1) * (nj - 1) * nk
                   for ni, nj, nk in (b.dims for b in c.blocks))
    return interior_cells(c)


def kernel_times(s, ki):
    """One iteration with CUDA events around every launch: {kernel: (ms, launches)}."""
    lib = s.lib
    ms = (C.c_double * abi.TRANS_NKCLASS)()
    nl = (C.c_int * abi.TRANS_NKCLASS)()
    rc = lib.trans_kernel_times(s.ctx, ki, ms, nl, abi.TRANS_NKCLASS)
    if rc != 0:
        raise RuntimeError(f"trans_kernel_times failed {rc}")
    return {lib.trans_kernel_class(k).decode(): (ms[k], nl[k]) for k in range(abi.TRANS_NKCLASS) if nl[k] > 0}


def pinned_copy(arr):
    """A page-locked host copy of a Fortran array (the caller's buffers in the end-to-end leg)."""
    import torch
    t = torch.empty(arr.size, dtype=torch.float64, pin_memory=True)
    out = t.numpy().reshape(arr.shape, order="F")
    out[...] = arr
    return out, t


def run_e2e(s, c, st, ki0, steps):
    """Per step through the C ABI with host buffers: upload the state (V, PP, T, Rmiu, Wt0,
    Wt1 as the Fortran caller holds them, page-locked) with trans_set_fields, iterate, download
    V, PP, T, Rmiu and the norms with trans_get_fields."""
    lib = s.lib
    keep = []
    up, down = [], []
    h2d = d2h = 0
    for ib, b in enumerate(c.blocks):
        for name in STATE_FIELDS:
            a, t = pinned_copy(CS.fortran_view(name, st[b.id][name]))
            keep.append(t)
            up.append((ib, abi.FIELD_ID[name], a))
            h2d += a.nbytes
        for name in ("V", "PP", "T", "RMIU"):
            shape = abi.field_shape(name, *b.dims)
            a, t = pinned_copy(np.zeros(shape, order="F"))
            keep.append(t)
            down.append((ib, abi.FIELD_ID[name], a))
            d2h += a.nbytes
    nb = len(c.blocks)
    norms = (abi.TransNorms * nb)()
    d2h += C.sizeof(norms)
    dp = C.POINTER(C.c_double)

    def table(lst):      # the (block, field, array) lists as the arrays of trans_set/get_fields
        n = len(lst)
        ib, fid, ptr = (C.c_int * n)(), (C.c_int * n)(), (dp * n)()
        for q, (b, f, a) in enumerate(lst):
            ib[q], fid[q], ptr[q] = b, f, a.ctypes.data_as(dp)
        return n, ib, fid, ptr
    tu, td = table(up), table(down)
    lib.trans_sync(s.ctx)
    t0 = time.perf_counter()
    for q in range(steps):
        if lib.trans_set_fields(s.ctx, *tu) != 0:
            raise RuntimeError("trans_set_fields failed")
        rc = lib.trans_iterate(s.ctx, ki0 + q, norms)
        if rc != 0:
            raise RuntimeError(f"iterate failed {rc}")
        if lib.trans_get_fields(s.ctx, *td) != 0:
            raise RuntimeError("trans_get_fields failed")
    lib.trans_sync(s.ctx)
    dt = time.perf_counter() - t0
    return dt, h2d, d2h


def cpu_sample(c, conns, geo, st, seconds=15.0):
    """The oracle on the host cores for a bounded number of iterations of the same workload."""
    from oracle.oracle import OracleSolver, load
    load().oracle_set_threads(1)
    o = OracleSolver(c, conns, geo, st)
    o.iterate(1)
    n, t0 = 0, time.perf_counter()
    while True:
        o.iterate(2 + n)
        n += 1
        if time.perf_counter() - t0 > seconds or n >= 50:
            break
    dt = time.perf_counter() - t0
    return interior_cells(c) * sub_iterations(c) * n / dt / 1e6, n, dt


def reference_arm(args):
    """--impl reference: the reference algorithm on the host cores (oracle, OpenMP over blocks)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    c, conns, geo, st = make_case(args.case, "fp64", args.nk)
    from oracle.oracle import OracleSolver, load
    threads = load().oracle_set_threads(os.cpu_count() or 1)
    o = OracleSolver(c, conns, geo, st)
    for w in range(args.warmup):
        o.iterate(1 + w)
    t0 = time.perf_counter()
    for q in range(args.steps):
        o.iterate(1 + args.warmup + q)
    dt = time.perf_counter() - t0
    ncell = interior_cells(c)
    v = ncell * sub_iterations(c) * args.steps / dt / 1e6
    line = {"metric": "Mcell-iter/s", "value": v, "unit": "Mcell-iter/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": c.name, "cells": ncell, "blocks": len(c.blocks), "precision": "fp64",
                       "implementation": "C++ FP64 restatement of the reference (oracle/), OpenMP over blocks"},
            "cpu_baseline": {"value": v, "unit": "Mcell-iter/s", "cores": min(threads, len(c.blocks)),
                             "kind": "port",
                             "sample": f"{args.steps} iterations of {c.name}, OpenMP over its {len(c.blocks)} blocks "
                                       f"({threads} threads available)"},
            "e2e": {"value": v, "unit": "Mcell-iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def batched_leg(c, conns, geo, st, args):
    """N copies of the workload with back-pressure ratios spread over [0.80, 0.92] in one
    mixed-precision batch context (every kernel one launch for all of them): aggregate
    cell-iterations/s, timed like the single case (CUDA events, iteration graphs replayed)."""
    import copy
    from trans_gb300.solver import Batch
    prec = abi.TRANS_MIXED
    bt = Batch(prec)
    ratio0 = c.meta.get("p_ratio", 0.85)
    n = args.batch
    for q in range(n):
        cq = copy.copy(c)
        cq.params = CS.params_copy(c.params)
        ratio = 0.80 + 0.12 * q / max(n - 1, 1)
        cq.params.Pouthub = c.params.Pouthub * ratio / ratio0
        if bt.add(cq, conns, geo, st) is None:
            raise RuntimeError("batch does not fit")
    bt.iterate(max(args.warmup, 1))
    if bt.lib.trans_prepare(bt.ctx, -1) != 0:
        raise RuntimeError(bt.lib.trans_last_error(bt.ctx).decode())
    ms = C.c_double()
    rc = bt.lib.trans_batch_time_iterations(bt.ctx, args.steps, C.byref(ms))
    if rc != 0:
        raise RuntimeError(f"batched timing failed {rc}")
    ncell = interior_cells(c) * n
    out = {"cases": n, "cells": ncell, "value": ncell * sub_iterations(c) * args.steps / (ms.value * 1e-3) / 1e6,
           "unit": "Mcell-iter/s", "ms_per_step": ms.value / args.steps, "precision": "mixed",
           "device_gb": bt.bytes_in_use() / 1e9, "sweep_schedule": bt.lib.trans_tuning(bt.ctx).decode()[:40]}
    bt.close()
    return out


def batch_levels_arm(args):
    """Batched steady solves of uneven size: cascades at three grid levels (counts
    `--batch-levels C,M,F` of coarse ~0.35 M / medium 1.36 M / fine ~5.5 M cells), back-pressure
    ratios U[0.80, 0.92] and inlet angles from {36, 40, 44} deg (seeded; the angle rotates the
    grid, so each level's geometry is computed once per angle), all in one batch context under
    the device budget; aggregate cell-iterations/s timed like the single case."""
    from trans_gb300 import serving
    from trans_gb300.solver import Batch, device_block_metrics
    prec = abi.TRANS_MIXED if args.precision == "mixed" else abi.TRANS_FP64
    counts = [int(x) for x in args.batch_levels.split(",")]
    rng = np.random.default_rng(0)
    bt = Batch(prec, budget_bytes=int(args.budget_gb * 1e9))
    geoms, admitted, refused, cells = {}, 0, 0, 0
    t0 = time.perf_counter()
    for level, n in zip(("coarse", "medium", "fine"), counts):
        for q in range(n):
            ratio = float(rng.uniform(0.80, 0.92))
            angle = float(rng.choice([36.0, 40.0, 44.0]))
            kw = dict(serving.LEVELS[level])
            kw.update(serving.RAMP)
            key = (level, angle)
            c = cases.cascade(inflow_deg=angle, p_ratio=ratio, precision=prec, **kw)
            if key not in geoms:
                conns, geo = CS.compute_geometry(c, metrics_fn=device_block_metrics(bt.lib))
                geoms[key] = (conns, geo, CS.initial_state(c, geo, Q_dst=c.meta.get("Q_dst", 0.01)))
            conns, geo, st = geoms[key]
            if bt.add(c, conns, geo, st) is None:
                refused += 1
                continue
            admitted += 1
            cells += interior_cells(c)
    setup_s = time.perf_counter() - t0
    geoms.clear()
    bt.iterate(max(args.warmup, 1))
    if bt.lib.trans_prepare(bt.ctx, -1) != 0:
        raise RuntimeError(bt.lib.trans_last_error(bt.ctx).decode())
    ms = C.c_double()
    rc = bt.lib.trans_batch_time_iterations(bt.ctx, args.steps, C.byref(ms))
    if rc not in (0, abi.TRANS_E_NAN):
        raise RuntimeError(f"batched timing failed {rc}")
    value = cells * args.steps / (ms.value * 1e-3) / 1e6
    line = {"metric": "Mcell-iter/s", "value": value, "unit": "Mcell-iter/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms.value / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if prec == abi.TRANS_FP64 else "f32-flux/f64-update", "data": "synthetic",
            "config": {"workload": "batched cascades at three grid levels", "requested": counts, "admitted": admitted,
                       "refused_over_budget": refused, "cells": cells, "budget_gb": args.budget_gb,
                       "device_gb_in_use": bt.bytes_in_use() / 1e9, "host_setup_s": setup_s,
                       "sweep_schedule": bt.lib.trans_tuning(bt.ctx).decode()[:60]},
            "nan_in_timed_steps": rc == abi.TRANS_E_NAN}
    bt.close()
    print(json.dumps(line))


def serve_arm(args):
    """Serving stream: seeded Poisson arrivals of cascade solves (grid level coarse 60% /
    medium 30% / fine 10%, back-pressure ratio U[0.80,0.92], inlet Mach U[0.5,0.7]) admitted
    into one batch context under a device-memory budget, each retired at its residual drop."""
    from trans_gb300 import serving
    prec = abi.TRANS_MIXED if args.precision == "mixed" else abi.TRANS_FP64
    reqs = serving.poisson_requests(rate=args.rate, duration=args.duration, seed=0)
    rep = serving.serve(reqs, precision=prec, budget_bytes=int(args.budget_gb * 1e9), drop=args.drop,
                        max_iters=20000)
    recs = rep.pop("records")
    by_level = {}
    for r in recs:
        by_level.setdefault(r.level, []).append(r.iterations)
    line = {"metric": "p50/p99 solve latency", "value": rep["latency_p50_s"], "unit": "s",
            "p99": rep["latency_p99_s"], "throughput_mcell_iter_s": rep["throughput_mcell_iter_s"],
            "higher_is_better": False, "n_gpus": 1, "dtype": "f64" if prec == abi.TRANS_FP64 else "f32-flux/f64-update",
            "data": "synthetic",
            "config": {"workload": "serving stream", "rate_per_s": args.rate, "duration_s": args.duration,
                       "retire_at_drop": args.drop, "budget_gb": args.budget_gb,
                       "mix": "coarse 0.6 / medium 0.3 / fine 0.1", "requests": rep["requests"]},
            "completed": rep["completed"], "converged": rep["converged"], "wall_s": rep["wall_s"],
            "iterations_by_level": {k: [min(v), int(np.median(v)), max(v)] for k, v in by_level.items()},
            "setup_s_median_by_level": rep["setup_s_by_level"],
            "loss_by_level": {lv: [round(r.integrals["loss"], 5) for r in recs if r.level == lv and r.integrals]
                              for lv in by_level}}
    print(json.dumps(line))


def roofline(lib, c, kt, nsub, precision, sched):
    """Roofline of the dominant kernel class from per-launch CUDA-event times of one iteration:
    algorithmic bytes per launch / launch time against the measured HBM copy bandwidth, and the
    binding roof where it is not HBM (the FP64 pipe of the FP64 face fluxes, the dependent-step
    latency of the hyperplane sweeps)."""
    pk = peaks()
    hbm = pk.get("hbm_gbs", FALLBACK_HBM)
    fp64 = lib.trans_probe_fma_gflops(1)
    fp32 = lib.trans_probe_fma_gflops(0)
    dom = max(kt, key=lambda k: kt[k][0])
    dom_ms, dom_n = kt[dom]
    per_launch_ms = dom_ms / dom_n
    nunit = units(c, dom) * nsub
    word = 4.0 if precision == "mixed" and dom in FP32_KERNELS else 8.0
    alg_bytes = ALG_WORDS.get(dom, 0) * word * nunit / dom_n
    achieved = alg_bytes / (per_launch_ms * 1e-3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": None, "kernel": dom, "launches_per_step": dom_n, "ms_per_launch": per_launch_ms,
            "alg_bytes_per_launch": alg_bytes,
            "peak_source": "measured" if "hbm_gbs" in pk else "fallback",
            "fp64_pipe_gflops_peak_measured": fp64, "fp32_pipe_gflops_peak_measured": fp32}
    if dom == "k_face_flux" and precision == "fp64":
        # the binding roof of the FP64 residual is the FP64 pipe: thread-instructions per second
        # against the probe's FMA rate (one FMA = one FP64 thread-instruction)
        inst = FACE_FP64_INST * nunit / dom_n / (per_launch_ms * 1e-3)
        roof["binding"] = "fp64_pipe"
        roof["fp64_inst_per_s"] = inst
        roof["fp64_pipe_frac"] = inst / (fp64 * 1e9 / 2.0)
        roof["traffic"] = FACE_DRAM_BYTES * nunit / dom_n
        roof["traffic_source"] = FACE_DRAM_SOURCE
    elif dom == "k_sweep":
        # the sweeps are bound by one dependent step per i+j+k hyperplane (per two with the mixed
        # path's two-plane launches): report the measured step against the floor of a dependent
        # launch chain of the same width (graph replay)
        pairs = sched.startswith("sweep=pairs")
        roof["binding"] = "latency (one dependent step per " + ("two i+j+k hyperplanes" if pairs else "i+j+k hyperplane") + ")"
        if sched.startswith("sweep=planes") or pairs:
            cells_per_plane = interior_cells(c) * nsub * 2 / dom_n      # dom_n counts both sweeps' launches
            # threads per launch: 8 per position in the FP64 path, 1 in the mixed path, 4 per
            # second-plane position (half a launch's positions) in the two-plane launches
            threads = cells_per_plane * (8 if precision == "fp64" else (2 if pairs else 1))
            grid = max(1, int(round(threads / 128)))
            chained = "chained" in sched.split(";")[0] or "early" in sched.split(";")[0]
            floor_us = lib.trans_probe_chain_us(1 if chained else 0, grid)
            roof["latency"] = {"us_per_step": per_launch_ms * 1e3, "floor_us_per_step": floor_us,
                               "frac": floor_us / (per_launch_ms * 1e3) if floor_us > 0 else None,
                               "floor": f"dependent launch chain, {grid} CTAs x 128 threads, one L2 round trip per step"}
    return roof


def measure(c, conns, geo, st, precision, args, world):
    """One context of the workload in `precision`: W warm-up steps (the last with CUDA events
    around every stage), trans_prepare (untimed tuning and graph capture), K steps timed with
    CUDA events on the context's stream, clocks sampled meanwhile; then the end-to-end leg
    through the C ABI with page-locked host buffers and the per-kernel times of one more step."""
    p = CS.params_copy(c.params)
    p.precision = abi.TRANS_MIXED if precision == "mixed" else abi.TRANS_FP64
    s = Solver(c, conns, geo, st, params=p)
    lib = s.lib
    ncell, nsub = interior_cells(c), sub_iterations(c)
    ki = 1
    for _ in range(max(args.warmup - 1, 0)):
        s.iterate(ki); ki += 1
    stage_ms = (C.c_double * len(abi.STAGES))()
    lib.trans_stage_times(s.ctx, ki, stage_ms); ki += 1
    if lib.trans_prepare(s.ctx, ki) != 0:
        raise RuntimeError(f"trans_prepare failed: {lib.trans_last_error(s.ctx)}")
    launches0 = lib.trans_kernel_launches(s.ctx)
    clk = ClockSampler()
    clk.start()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    ms = time_resident(s, ki, args.steps)
    ki += args.steps
    launches = lib.trans_kernel_launches(s.ctx) - launches0
    clocks = clk.stop()
    ms = max_over_ranks(ms, world)
    value = replica_rate(ncell * nsub * args.steps, ms * 1e-3, world)
    e2e_steps = max(2, min(args.steps, 10))
    dt, h2d, d2h = run_e2e(s, c, st, ki, e2e_steps)
    ki += e2e_steps
    e2e = replica_rate(ncell * nsub * e2e_steps, max_over_ranks(dt, world), world)
    kt = kernel_times(s, ki)
    sched = lib.trans_tuning(s.ctx).decode()
    out = {"value": value, "unit": "Mcell-iter/s", "ms_per_step": ms / args.steps,
           "e2e": {"value": e2e, "unit": "Mcell-iter/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
           "gpu_launches": int(launches), "clocks": clocks,
           "roofline": roofline(lib, c, kt, nsub, precision, sched),
           "stage_ms": {n: stage_ms[i] for i, n in enumerate(abi.STAGES)},
           "kernel_ms": {k: round(v[0], 4) for k, v in sorted(kt.items(), key=lambda x: -x[1][0])},
           "device_gb": lib.trans_device_bytes(s.ctx) / 1e9, "sweep_schedule": sched}
    s.close()
    return out


def serving_leg(args):
    """Bounded serving stream (mixed precision): seeded Poisson arrivals at `--rate` per second
    for `--duration` seconds, grid level coarse 60% / medium 30% / fine 10%, back-pressure ratio
    U[0.80, 0.92], inlet Mach U[0.5, 0.7], admission under a `--budget-gb` device budget, each
    request retired at a `--drop` residual drop or after `--max-iters` iterations."""
    from trans_gb300 import serving
    reqs = serving.poisson_requests(rate=args.rate, duration=args.duration, seed=0)
    rep = serving.serve(reqs, precision=abi.TRANS_MIXED, budget_bytes=int(args.budget_gb * 1e9), drop=args.drop,
                        max_iters=args.max_iters, prep_workers=args.prep_workers)
    recs = rep.pop("records")
    by_level = {}
    for r in recs:
        by_level.setdefault(r.level, []).append(r.iterations)
    return {"p50_s": rep["latency_p50_s"], "p99_s": rep["latency_p99_s"], "unit": "s",
            "throughput_mcell_iter_s": rep["throughput_mcell_iter_s"], "precision": "mixed",
            "rate_per_s": args.rate, "duration_s": args.duration, "retire_at_drop": args.drop,
            "max_iters": args.max_iters, "budget_gb": args.budget_gb, "mix": "coarse 0.6 / medium 0.3 / fine 0.1",
            "requests": rep["requests"], "completed": rep["completed"], "converged": rep["converged"],
            "hit_iteration_cap": sum(r.status == "max_iters" for r in recs),
            "nan": sum(r.status == "nan" for r in recs), "wall_s": rep["wall_s"],
            "iterations_by_level": {k: [min(v), int(np.median(v)), max(v)] for k, v in by_level.items()},
            "setup_s_median_by_level": rep["setup_s_by_level"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--case", default=os.environ.get("TRANS_BENCH_CASE", "cascade"))
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"], help="precision of the headline value")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nk", type=int, default=64, help="spanwise cells of the cascade (64 = full size)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-precision leg")
    ap.add_argument("--batch-levels", default=None,
                    help="batched cascades at three grid levels: counts C,M,F (e.g. 32,24,8)")
    ap.add_argument("--batch", type=int, default=8,
                    help="copies of the workload (back-pressure ratios 0.80..0.92) in one mixed batch context (0: none)")
    ap.add_argument("--serve", action="store_true", help="run only the serving stream (p50/p99 latency)")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg")
    ap.add_argument("--rate", type=float, default=4.0, help="serving: Poisson arrivals per second")
    ap.add_argument("--duration", type=float, default=SERVE_DURATION, help="serving: seconds of arrivals")
    ap.add_argument("--drop", type=float, default=SERVE_DROP, help="serving: residual drop at which a request retires")
    ap.add_argument("--max-iters", type=int, default=SERVE_MAX_ITERS, help="serving: iteration cap of a request")
    ap.add_argument("--prep-workers", type=int, default=4, help="serving: host set-up threads")
    ap.add_argument("--budget-gb", type=float, default=150.0, help="serving: device-memory budget")
    args = ap.parse_args()
    if args.batch_levels:
        return batch_levels_arm(args)
    if args.serve:
        return serve_arm(args)
    if args.impl == "reference":
        return reference_arm(args)
    rank, world = init_replicas()
    from trans_gb300.solver import device_block_metrics
    c, conns, geo, st = make_case(args.case, "fp64", args.nk, metrics_fn=device_block_metrics())
    ncell = interior_cells(c)
    nsub = sub_iterations(c)
    head = measure(c, conns, geo, st, args.precision, args, world)
    line = {
        "metric": "Mcell-iter/s", "value": head["value"], "unit": "Mcell-iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32-flux/f64-update",
        "data": "synthetic",
        "config": {"workload": c.name, "cells": ncell, "blocks": len(c.blocks),
                   "block_nodes": [list(b.dims) for b in c.blocks], "precision": args.precision,
                   "sub_iterations_per_step": nsub,
                   "l2": f"working set {head['device_gb']:.2f} GB > L2 (no flush needed)",
                   "sweep_schedule": head["sweep_schedule"]},
        "e2e": head["e2e"], "gpu_launches": head["gpu_launches"], "clocks": head["clocks"],
        "roofline": head["roofline"], "stage_ms": head["stage_ms"], "kernel_ms": head["kernel_ms"],
    }
    if not args.no_mixed and args.precision == "fp64":
        m = measure(c, conns, geo, st, "mixed", args, world)
        m["vs_fp64"] = m["value"] / head["value"]
        m["e2e_vs_fp64"] = m["e2e"]["value"] / head["e2e"]["value"]
        line["mixed"] = m
    if args.batch > 1:
        b = batched_leg(c, conns, geo, st, args)
        b["vs_fp64"] = b["value"] / head["value"]
        line["batched"] = b
    if rank == 0 and not args.no_serve and world == 1:
        line["serving"] = serving_leg(args)
    if rank == 0 and not args.no_cpu:
        v, n, dt2 = cpu_sample(c, conns, geo, st)
        line["cpu_baseline"] = {"value": v, "unit": "Mcell-iter/s", "cores": 1, "kind": "port",
                                "sample": f"{n} iterations of {c.name} on one core ({dt2:.1f} s)"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
