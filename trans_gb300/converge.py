"""Run a case to a residual drop through the C ABI and report the convergence history, the
iteration count, the throughput and the integrated quantities (trans_gb300.integrals).

    python -m trans_gb300.converge --case cascade --precision mixed --drop 1e-6 --max-iters 20000
    python -m trans_gb300.converge --case cascade --level coarse --scheme muscl_roe --compare
    python -m trans_gb300.converge --case channel_walls --laminar --Re 1e4 --compare

With --compare both precisions run on the same case and the relative differences of the
mixed-precision results from the FP64 ones are reported (mass flow, total-pressure loss, blade
loading, wall force, field L-inf).  Output: one JSON object on stdout.
"""
import argparse
import json
import time

import numpy as np

from . import abi
from . import case as CS
from . import cases
from . import integrals
from .solver import Batch, global_residual


SCHEMES = {"mdcd_ausmpw": dict(Kind_Spatial=3, Kind_Roe=3), "muscl_roe": dict(Kind_Spatial=2, Kind_Roe=1),
           "muscl2_roe": dict(Kind_Spatial=1, Kind_Roe=1),
           "muscl_roe_wd2006": dict(Kind_Spatial=2, Kind_Roe=1, Kind_Model=2),
           "muscl_roerot": dict(Kind_Spatial=2, Kind_Roe=2)}
LEVELS = {"coarse": dict(ns=60, nh=32, nk=32), "medium": dict(nk=32), "full": dict()}


def make(name, precision, **kw):
    if name == "channel":
        c = cases.channel_bump(precision=precision, **kw)
    elif name == "channel_walls":          # no-slip walls on both sides instead of a far field
        c = cases.channel_bump(precision=precision, top=1, **kw)
    elif name == "cascade":
        c = cases.cascade(precision=precision, **kw)
    else:
        raise SystemExit(f"unknown case {name}")
    conns, geo = CS.compute_geometry(c)
    st = CS.initial_state(c, geo, Q_dst=c.meta.get("Q_dst", 0.01))
    return c, conns, geo, st


def run(name, precision, drop=1e-6, max_iters=20000, chunk=50, **kw):
    """Iterate in chunks (whole chunks replayed as CUDA graphs) until the global residual has
    dropped by `drop` from its first iteration or `max_iters` is reached."""
    c, conns, geo, st = make(name, precision, **kw)
    ncell = int(sum(np.prod([d - 1 for d in b.dims]) for b in c.blocks))
    bt = Batch(precision)
    cid = bt.add(c, conns, geo, st)
    hist = []
    t0 = time.perf_counter()
    g0 = None
    status = "max_iters"
    while True:
        it_done = bt.norms(cid)[0]
        if it_done >= max_iters:
            break
        n = 1 if g0 is None else min(chunk, max_iters - it_done)
        nan = bt.iterate(n)
        it, first, last = bt.norms(cid)
        g = global_residual(last, c.blocks)
        if g0 is None:
            g0 = global_residual(first, c.blocks)
        hist.append((it, g / g0))
        if nan or not np.isfinite(g):
            status = "nan"
            break
        if g <= drop * g0:
            status = "converged"
            break
    wall = time.perf_counter() - t0
    it = bt.norms(cid)[0]
    fields = [{f: bt.get_field(cid, ib, f) for f in ("V", "PP", "T", "RMIU")} for ib in range(len(c.blocks))]
    bt.close()
    return {"case": c.name, "precision": "mixed" if precision == abi.TRANS_MIXED else "fp64", "status": status,
            "iterations": it, "drop": hist[-1][1] if hist else None, "wall_s": wall,
            "mcell_iter_s": ncell * it / wall / 1e6, "cells": ncell, "history": hist}, (c, conns, geo, fields)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="cascade")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--drop", type=float, default=1e-6)
    ap.add_argument("--max-iters", type=int, default=20000)
    ap.add_argument("--chunk", type=int, default=50)
    ap.add_argument("--compare", action="store_true", help="run FP64 and mixed and report their differences")
    ap.add_argument("--nk", type=int, default=None, help="spanwise cells of the cascade")
    ap.add_argument("--level", default=None, choices=sorted(LEVELS), help="cascade grid level")
    ap.add_argument("--scheme", default=None, choices=sorted(SCHEMES), help="reconstruction + flux")
    ap.add_argument("--laminar", action="store_true", help="laminar (IF_Turb_org = 0)")
    ap.add_argument("--Re", type=float, default=None, help="channel Reynolds number Re_L")
    args = ap.parse_args()
    kw = dict(LEVELS[args.level]) if args.level else {}
    if args.nk is not None:
        kw["nk"] = args.nk
    if args.scheme:
        kw.update(SCHEMES[args.scheme])
    if args.laminar:
        kw["IF_Turb_org"] = 0
    if args.Re is not None:
        kw["Re_L"] = args.Re
    if args.compare:
        r64, s64 = run(args.case, abi.TRANS_FP64, args.drop, args.max_iters, args.chunk, **kw)
        r32, s32 = run(args.case, abi.TRANS_MIXED, args.drop, args.max_iters, args.chunk, **kw)
        c, conns, geo, f64 = s64
        err = integrals.error_table(c, conns, geo, s32[3], f64)
        out = {"fp64": r64, "mixed": r32, "mixed_vs_fp64": err,
               "speedup_time_to_drop": r64["wall_s"] / r32["wall_s"] if r32["wall_s"] > 0 else None}
    else:
        prec = abi.TRANS_MIXED if args.precision == "mixed" else abi.TRANS_FP64
        out, (c, conns, geo, f) = run(args.case, prec, args.drop, args.max_iters, args.chunk, **kw)
        out["integrals"] = {k: v for k, v in integrals.summary(c, conns, geo, f).items() if k != "cp_blade"}
    print(json.dumps(out, default=float))


if __name__ == "__main__":
    main()
