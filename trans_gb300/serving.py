"""Serving loop: steady cascade solves of different back pressures, inlet Mach numbers and grid
sizes arrive as requests, are admitted into one batch context as device memory allows, iterate
together (every kernel launch covers all resident cases) and retire individually at their
residual drop.  Continuous batching: requests that arrive while others are on the GPU join at
the next iteration, and a retired case frees its memory for the queue at once.

Latency of a request = retirement time - arrival time (queueing, host set-up of the grid and
geometry, and the solve).  Throughput = cell-iterations of all cases / wall time.

  reqs = poisson_requests(rate=4.0, duration=60.0, seed=0)
  rep = serve(reqs, precision=abi.TRANS_MIXED, budget_bytes=150e9)
"""
import math
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from . import abi
from . import case as CS
from . import cases
from .solver import Batch, device_block_metrics, global_residual

# grid levels of the cascade topology: (ns, nr, nh, nk) for about 0.35 M, 1.36 M and 5.4 M cells
# grid levels: coarse ~0.35 M, medium 1.36 M, fine ~5.5 M cells.  The fine level also doubles the
# leading/trailing-edge caps and blends the side clustering with uniform spacing: with the
# medium level's cosine clustering at 240 side cells, the side cell next to the trailing-edge
# cap is 1/60 of the cap cell and the solve diverged at the trailing-edge/endwall corner
LEVELS = {"coarse": dict(ns=60, nh=32, nk=32), "medium": dict(),
          "fine": dict(ns=240, nh=128, nk=128, nle=16, nte=8, cluster=0.6)}
# CFL ramp of every request (Time/SpectralRadius.F90:159-160: CFL_sub grows linearly from
# CFL_Sub_start to CFL_Sub_end over CFL_Sub_step iterations); an impulsive start at CFL 10
# diverged on the fine level
RAMP = dict(CFL_Sub_start=2.0, CFL_Sub_end=10.0, CFL_Sub_step=200)


@dataclass
class Request:
    rid: int
    arrival: float                     # seconds after the start of the stream
    level: str = "coarse"
    p_ratio: float = 0.85
    mach: float = 0.6
    grid: dict = field(default_factory=dict)   # overrides of the cascade generator (tests)
    # filled in by the loop
    admitted: float = math.nan
    retired: float = math.nan
    iterations: int = 0
    drop: float = math.nan
    status: str = "queued"
    cells: int = 0
    result: dict = None
    integrals: dict = None             # mass flow, loss, wall forces at retirement (on the device)
    setup_s: float = math.nan          # host set-up (grid, geometry, initial field)


def poisson_requests(rate=4.0, duration=60.0, seed=0, mix=(("coarse", 0.6), ("medium", 0.3), ("fine", 0.1)),
                     p_ratio=(0.80, 0.92), mach=(0.5, 0.7)):
    """Poisson arrivals at `rate` per second over `duration` seconds (seeded): grid level drawn
    from `mix`, back-pressure ratio and inlet Mach number uniform in the given ranges."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    names = [m[0] for m in mix]
    probs = np.array([m[1] for m in mix], float)
    probs /= probs.sum()
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        out.append(Request(len(out), t, str(rng.choice(names, p=probs)), float(rng.uniform(*p_ratio)),
                           float(rng.uniform(*mach))))
    return out


def build_case(req, precision, metrics_fn=None):
    """Set-up of one request: grid, connectivity, geometry (the block metrics and wall
    distance by metrics_fn: on the GPU when given, else on the host) and initial field; records
    its duration in req.setup_s."""
    t0 = time.perf_counter()
    kw = dict(LEVELS.get(req.level, {}))
    kw.update(RAMP)
    kw.update(req.grid)
    c = cases.cascade(XM=req.mach, p_ratio=req.p_ratio, precision=precision, **kw)
    conns, geo = CS.compute_geometry(c, metrics_fn=metrics_fn)
    st = CS.initial_state(c, geo, Q_dst=c.meta.get("Q_dst", 0.01))
    req.setup_s = time.perf_counter() - t0
    return c, conns, geo, st


def serve(requests, precision=abi.TRANS_MIXED, budget_bytes=0, drop=1.0e-6, max_iters=20000, prep_workers=2,
          keep_fields=False, lib=None, time_limit=None, device_setup=True):
    """Run the request stream to completion (or until `time_limit` seconds); returns a report
    with p50/p99 latency, throughput and the per-request records.

    A request is admitted as soon as its host set-up is done and its device bytes fit the
    budget (later, smaller requests may pass a large one that does not fit yet); it retires
    when its global residual (block RMS norms of TIME_Update_V aggregated over blocks) has
    dropped by `drop` from its first iteration, after `max_iters` iterations, or on a NaN."""
    bt = Batch(precision, budget_bytes, lib)
    metrics_fn = device_block_metrics(bt.lib) if device_setup else None
    pending = sorted(requests, key=lambda r: r.arrival)
    prepping, ready, active = {}, [], {}
    done = []
    cell_iters = 0
    t0 = time.perf_counter()

    def now():
        return time.perf_counter() - t0

    def retire(cid, status):
        r, c = active.pop(cid)
        it, first, last = bt.norms(cid)
        r.iterations = it
        g0, g1 = global_residual(first, c.blocks), global_residual(last, c.blocks)
        r.drop = g1 / g0 if g0 > 0 else math.nan
        if status != "nan":
            r.integrals = bt.integrals(cid)
        if keep_fields:
            r.result = {ib: {f: bt.get_field(cid, ib, f) for f in ("V", "PP", "T", "RMIU")} for ib in range(len(c.blocks))}
        bt.remove(cid)
        r.retired = now()
        r.status = status
        done.append(r)

    with ThreadPoolExecutor(max_workers=prep_workers) as ex:
        while pending or prepping or ready or active:
            if time_limit is not None and now() > time_limit:
                break
            t = now()
            while pending and pending[0].arrival <= t:
                r = pending.pop(0)
                prepping[r.rid] = (r, ex.submit(build_case, r, precision, metrics_fn))
            for rid in sorted(prepping):
                r, f = prepping[rid]
                if f.done():
                    ready.append((r, f.result()))
                    del prepping[rid]
            ready.sort(key=lambda x: x[0].arrival)
            for item in list(ready):
                r, (c, conns, geo, st) = item
                cid = bt.add(c, conns, geo, st)
                if cid is None:
                    if not active:              # cannot fit even alone: refuse it
                        r.status = "refused"
                        r.retired = now()
                        done.append(r)
                        ready.remove(item)
                    continue
                r.admitted = now()
                r.cells = int(sum(np.prod([d - 1 for d in b.dims]) for b in c.blocks))
                r.status = "running"
                active[cid] = (r, c)
                ready.remove(item)
            if not active:
                nxt = pending[0].arrival - now() if pending else 0.005
                time.sleep(min(max(nxt, 0.0005), 0.005))
                continue
            bt.iterate(1)                       # a NaN case is retired below by its nan_flag
            for cid in list(active):
                r, c = active[cid]
                cell_iters += r.cells
                it, first, last = bt.norms(cid)
                if any(n["nan_flag"] for n in last):
                    retire(cid, "nan")
                    continue
                g0, g1 = global_residual(first, c.blocks), global_residual(last, c.blocks)
                if g0 > 0 and g1 <= drop * g0:
                    retire(cid, "converged")
                elif it >= max_iters:
                    retire(cid, "max_iters")
    wall = now()
    bt.close()
    lat = np.array([r.retired - r.arrival for r in done if r.status in ("converged", "max_iters")])
    return {
        "requests": len(requests), "completed": len(done),
        "converged": sum(r.status == "converged" for r in done),
        "latency_p50_s": float(np.percentile(lat, 50)) if lat.size else None,
        "latency_p99_s": float(np.percentile(lat, 99)) if lat.size else None,
        "latency_mean_s": float(lat.mean()) if lat.size else None,
        "setup_s_by_level": {lv: float(np.median([r.setup_s for r in done if r.level == lv]))
                             for lv in sorted({r.level for r in done}) if any(r.level == lv for r in done)},
        "wall_s": wall, "cell_iters": int(cell_iters),
        "throughput_mcell_iter_s": cell_iters / wall / 1e6 if wall > 0 else 0.0,
        "records": done,
    }
