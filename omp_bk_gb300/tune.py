"""Autotuner of the mixed-order persistent launch.

The launch runs every tile with the same block, whose threads are the
largest tile's lines (elements x (p+1)^2): tiles of the other orders should
have about as many lines, or threads idle in their sweeps.  So the tuner
picks one line budget T for the whole plan and gives order p
max(1, T // (p+1)^2) elements per tile; every candidate T is timed with CUDA
events on the plan itself (element counts capped), the fastest kept.
Results are cached per GPU name, precision, kernel body and order set in a
JSON file (~/.cache/omp_bk_gb300/tune.json, or $BK_TUNE_CACHE)."""
from __future__ import annotations

import json
import os

from . import PREC_MIXED
from .helmholtz import HelmholtzPlan

CACHE = os.environ.get("BK_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "omp_bk_gb300", "tune.json"))

LINE_BUDGETS = (64, 96, 128, 160, 192, 256)


def tiles_for(p: int, lines: int) -> int:
    """Elements per tile of order p under a budget of `lines` threads."""
    return max(1, lines // (p + 1) ** 2)


def candidates(p: int):
    """The elements per tile the tuner can give order p."""
    return sorted({tiles_for(p, t) for t in LINE_BUDGETS})


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


def tune(orders, prec=PREC_MIXED, max_elements=65536, reps=5, use_cache=True, verbose=False, kernel=0):
    """{p: elements per tile} for the (p, E) orders, for the plan body
    `kernel` (KERNEL_AUTO: the plan's default)."""
    import torch
    ps = sorted(p for p, _ in orders)
    key = f"{torch.cuda.get_device_name()}|prec{prec}|kernel{kernel}|p{','.join(map(str, ps))}"
    cache = {}
    if use_cache and os.path.exists(CACHE):
        try:
            cache = json.load(open(CACHE))
        except (OSError, ValueError):
            cache = {}
    if key in cache:
        return {int(p): int(e) for p, e in cache[key].items()}
    capped = [(p, max(1, min(int(E), max_elements))) for p, E in orders]
    dt = torch.float64 if prec == 0 else torch.float32
    times = {}
    G = M = None
    for lines in LINE_BUDGETS:
        plan = HelmholtzPlan([(p, E, tiles_for(p, lines)) for p, E in capped])
        plan.set_kernel(kernel)
        if G is None:
            G, M = plan.geometry()
            G, M = G.to(dt), M.to(dt)
            u = torch.ones(plan.n, dtype=dt, device="cuda")
            v = torch.empty_like(u)
        times[lines] = _time(plan, G, M, u, v, prec, reps, torch)
        plan.close()
    best_lines = min(times, key=times.get)
    best = {p: tiles_for(p, best_lines) for p, _ in orders}
    if verbose:
        print("tune: " + ", ".join(f"{t}:{ms:.3f}ms" for t, ms in sorted(times.items())) + f" -> {best_lines} lines")
    if use_cache:
        cache[key] = {str(p): e for p, e in best.items()}
        try:
            os.makedirs(os.path.dirname(CACHE), exist_ok=True)
            json.dump(cache, open(CACHE, "w"), indent=1)
        except OSError:
            pass
    return best
