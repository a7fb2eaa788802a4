"""Autotuner of the mixed-order persistent launch: per order p, the number of
elements per tile (one tile = one block iteration; elements x (p+1)^2 threads
of the block's 256 are busy).  Every candidate is timed with CUDA events on a
single-order plan of the order's own size (capped), the fastest kept.
Results are cached per GPU name and precision in a JSON file
(~/.cache/omp_bk_gb300/tune.json, or $BK_TUNE_CACHE)."""
from __future__ import annotations

import json
import os

from . import PREC_MIXED
from .helmholtz import HelmholtzPlan

CACHE = os.environ.get("BK_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "omp_bk_gb300", "tune.json"))


def candidates(p: int):
    q2 = (p + 1) ** 2
    top = 256 // q2
    c = sorted({e for e in (1, 2, 3, 4, 6, 8, 12, 16, 24, 28) if e <= top} | {top})
    return [e for e in c if e >= 1]


def _time(plan, G, M, u, v, prec, reps, torch):
    plan.apply(G, M, 1.0, u, v, prec=prec)
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(reps):
        plan.apply(G, M, 1.0, u, v, prec=prec)
    t1.record()
    torch.cuda.synchronize()
    return t0.elapsed_time(t1) / reps


def tune(orders, prec=PREC_MIXED, max_elements=65536, reps=5, use_cache=True, verbose=False):
    """{p: elements per tile} for the (p, E) orders."""
    import torch
    key = f"{torch.cuda.get_device_name()}|prec{prec}"
    cache = {}
    if use_cache and os.path.exists(CACHE):
        try:
            cache = json.load(open(CACHE))
        except (OSError, ValueError):
            cache = {}
    got = cache.get(key, {})
    best = {}
    for p, E in orders:
        if str(p) in got:
            best[p] = int(got[str(p)])
            continue
        En = max(1, min(E, max_elements))
        dt = torch.float64 if prec == 0 else torch.float32
        times = {}
        for eb in candidates(p):
            plan = HelmholtzPlan([(p, En, eb)])
            G, M = plan.geometry()
            G, M = G.to(dt), M.to(dt)
            u = torch.ones(plan.n, dtype=dt, device="cuda")
            v = torch.empty_like(u)
            times[eb] = _time(plan, G, M, u, v, prec, reps, torch)
            plan.close()
            del G, M, u, v
        best[p] = min(times, key=times.get)
        got[str(p)] = best[p]
        if verbose:
            print(f"tune p={p}: " + ", ".join(f"{e}:{t:.3f}ms" for e, t in sorted(times.items())) + f" -> {best[p]}")
    if use_cache:
        cache[key] = got
        try:
            os.makedirs(os.path.dirname(CACHE), exist_ok=True)
            json.dump(cache, open(CACHE, "w"), indent=1)
        except OSError:
            pass
    return best
