"""Autotuner of the mixed-order persistent launch.

The persistent launch walks tiles of every order with one block shape.  The
choices that shape it are timed here with CUDA events on the plan itself
(element counts capped), the fastest kept:

* the block size B (threads per block of the even-odd sweep body), from
  BLOCKS;
* for FP32 storage, whether each tile's G is staged in shared memory by TMA
  or read in the pointwise stage straight from global memory (prefetched
  into L2 one tile ahead): staging costs shared memory and so blocks per SM,
  reading costs load latency;
* the elements per tile eb_p of every order p: a tile of eb_p elements has
  eb_p (p+1)^2 lines, which the block's B threads sweep (a tile with more
  lines than threads loops over them), and the largest tile's stages and
  work boxes set the launch's shared memory and so its blocks per SM.

Search: every (B, staging) starts from the tiles whose lines fill B best (at
most B lines); the best start is then improved one order at a time over the
counts whose lines fill 1..8 sweeps of B threads (coordinate descent, two
passes, each shape timed over 15 applies).  Shapes whose launch would not
fit a block's shared memory are skipped (tuning FP32 storage, the FP64
launch on the same tiles too: it runs the solver's residual unless given
its own shape).  The
column body (one thread per column, tiles of at most 256 columns) keeps one
line budget T for the plan, eb_p = max(1, T // (p+1)^2).

tune_apply() does the same for the single-order BK5 applies: per order it
times the two kernel shapes (one thread per line, one thread per k-column)
and sets the faster as the library's KERNEL_AUTO choice for that order,
precision, layout and mass term.

Results are cached per GPU name, precision, body and (capped) orders in a JSON file
(~/.cache/omp_bk_gb300/tune.json, or $BK_TUNE_CACHE)."""
from __future__ import annotations

import json
import os

from . import KERNEL_COLUMN, PREC_MIXED
from .helmholtz import HelmholtzPlan

CACHE = os.environ.get("BK_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "omp_bk_gb300", "tune.json"))

BLOCKS = (128, 192, 256)      # threads per block of the sweep body
GSTAGE = (0, 1)               # FP32 G read from global memory / staged
LINE_BUDGETS = (64, 96, 128, 160, 192, 256)   # column body
MAX_TILE_LINES = 1024         # bk_order_range: elems_per_tile * q^2 <= 1024
SWEEPS = 8                    # sweep-body tiles: lines for 1..SWEEPS sweeps of the block
MAX_SMEM = 232448             # shared memory of one block, bytes


def tiles_for(p: int, lines: int) -> int:
    """Elements per tile of order p under a budget of `lines` lines."""
    return max(1, lines // (p + 1) ** 2)


def candidates(p: int, block: int = 0):
    """Elements per tile the tuner tries for order p: with a block of
    `block` threads, the counts whose lines fill 1..SWEEPS sweeps of the
    block best (a tile's fixed costs, its staging and barriers, spread over
    more points per thread as it grows); without, the column body's line
    budgets."""
    if not block:
        return sorted({tiles_for(p, t) for t in LINE_BUDGETS})
    q2 = (p + 1) ** 2
    out = set()
    for k in range(1, SWEEPS + 1):
        eb = max(1, (k * block) // q2)
        if eb * q2 <= MAX_TILE_LINES:
            out.add(eb)
    return sorted(out)


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


class _Bench:
    """Times plans over the capped orders on one set of operator data."""

    def __init__(self, capped, prec, kernel, reps, torch):
        self.capped, self.prec, self.kernel, self.reps, self.torch = capped, prec, kernel, reps, torch
        self.dt = torch.float64 if prec == 0 else torch.float32
        self.data = None
        self.seen = {}

    def __call__(self, block, gstage, tiles):
        key = (block, gstage, tuple(sorted(tiles.items())))
        if key in self.seen:
            return self.seen[key]
        plan = HelmholtzPlan([(p, E, tiles[p]) for p, E in self.capped])
        try:
            plan.set_kernel(self.kernel)
            plan.set_shape(block, gstage)
            # FP32 storage: the plan's FP64 applies (the solver's residual)
            # run on the same tiles unless given their own (make_plan's
            # fp64), so both forms' stages must fit a block's shared memory
            need = plan.smem_bytes(fp64=True)
            if self.prec != 0:
                need = max(need, plan.smem_bytes(fp64=False))
            if need > MAX_SMEM:
                ms = float("inf")
            else:
                if self.data is None:
                    G, M = plan.geometry()
                    u = self.torch.ones(plan.n, dtype=self.dt, device="cuda")
                    self.data = (G.to(self.dt), M.to(self.dt), u, self.torch.empty_like(u))
                G, M, u, v = self.data
                ms = _time(plan, G, M, u, v, self.prec, self.reps, self.torch)
        finally:
            plan.close()
        self.seen[key] = ms
        return ms


def _search_sweep(bench, orders, prec, verbose):
    ps = [p for p, _ in orders]
    stages = GSTAGE if prec != 0 else (0,)
    # the best-filling tiles (at most B lines) for every block size and staging
    starts = {}
    for B in BLOCKS:
        for gs in stages:
            tiles = {p: tiles_for(p, B) for p in ps}
            starts[(B, gs)] = (bench(B, gs, tiles), tiles)
    B, gs = min(starts, key=lambda k: starts[k][0])
    best_ms, best = starts[(B, gs)]
    best = dict(best)
    for _ in range(2):
        changed = False
        for p in ps:
            for eb in candidates(p, B):
                if eb == best[p]:
                    continue
                trial = dict(best)
                trial[p] = eb
                ms = bench(B, gs, trial)
                if ms < best_ms:
                    best_ms, best, changed = ms, trial, True
        if not changed:
            break
    if verbose:
        print("tune (sweep body): starts " + ", ".join(f"B={b} g={g}:{starts[(b, g)][0]:.3f}ms" for b, g in starts) +
              f" -> B={B} gstage={gs} tiles {best} {best_ms:.3f}ms")
    return {"block": B, "gstage": gs, "tiles": best, "ms": best_ms,
            "starts_ms": {f"B{b}_g{g}": v[0] for (b, g), v in starts.items()}}


def _search_column(bench, orders, verbose):
    times = {}
    for lines in LINE_BUDGETS:
        times[lines] = bench(0, 0, {p: tiles_for(p, lines) for p, _ in orders})
    best_lines = min(times, key=times.get)
    if verbose:
        print("tune (column body): " + ", ".join(f"{t}:{ms:.3f}ms" for t, ms in sorted(times.items())) +
              f" -> {best_lines} lines")
    return {"block": 0, "gstage": 0, "tiles": {p: tiles_for(p, best_lines) for p, _ in orders},
            "ms": times[best_lines]}


def tune(orders, prec=PREC_MIXED, max_elements=65536, reps=15, use_cache=True, verbose=False, kernel=0):
    """The plan shape for the (p, E) orders and the plan body `kernel`
    (KERNEL_AUTO: the plan's default, the even-odd sweep body for GLL):
    {"block": threads per block (0: the largest tile's lines), "gstage": FP32
    G staged (1) or read from global memory (0), "tiles": {p: elements per
    tile}, "ms": the tuned plan's time on the capped orders}."""
    import torch
    capped = [(p, max(1, min(int(E), max_elements))) for p, E in orders]
    # the key holds the (capped) element counts: the best tiles depend on
    # the balance of the orders' work
    sig = ",".join(f"{p}:{E}" for p, E in sorted(capped))
    key = f"{torch.cuda.get_device_name()}|prec{prec}|kernel{kernel}|{sig}|v4"
    cache = {}
    if use_cache and os.path.exists(CACHE):
        try:
            cache = json.load(open(CACHE))
        except (OSError, ValueError):
            cache = {}
    if key in cache:
        c = cache[key]
        return {"block": int(c["block"]), "gstage": int(c["gstage"]),
                "tiles": {int(p): int(e) for p, e in c["tiles"].items()}, "ms": c.get("ms")}
    bench = _Bench(capped, prec, kernel, reps, torch)
    if kernel == KERNEL_COLUMN:
        res = _search_column(bench, capped, verbose)
    else:
        res = _search_sweep(bench, capped, prec, verbose)
    res["evaluated"] = len(bench.seen)
    if use_cache:
        cache[key] = {"block": res["block"], "gstage": res["gstage"],
                      "tiles": {str(p): e for p, e in res["tiles"].items()}, "ms": res["ms"]}
        try:
            os.makedirs(os.path.dirname(CACHE), exist_ok=True)
            json.dump(cache, open(CACHE, "w"), indent=1)
        except OSError:
            pass
    return res


def make_plan(orders, tuned, kernel=0, fp64=None):
    """A HelmholtzPlan over the (p, E) orders in the tuned shape; fp64: the
    shape tuned for FP64 storage (tune(prec=PREC_FP64)), given to the plan's
    FP64 launches (the solver's residual) apart from the FP32 ones."""
    plan = HelmholtzPlan([(p, E, tuned["tiles"][p]) for p, E in orders])
    if kernel:
        plan.set_kernel(kernel)
    plan.set_shape(tuned.get("block", 0), tuned.get("gstage", 0))
    if fp64 is not None and plan.kernel != KERNEL_COLUMN:
        plan.set_fp64_shape(fp64["tiles"], fp64.get("block", 0))
    return plan


# ---- single-order BK5 applies: the kernel shape per order ------------------------

def tune_apply(orders, prec=PREC_MIXED, layout=2, with_mass=True, reps=10, max_elements=65536, use_cache=True,
               verbose=False):
    """BK5's kernel shape per order for bk5_apply(..., kernel=KERNEL_AUTO):
    for every (p, E) of `orders` (E capped) the sweep kernel (one thread per
    line) and the column kernel (one thread per k-column) are timed with
    CUDA events on the same inputs, and the faster is set as AUTO's choice
    for (p, prec, layout, mass term) in the library (bk5_set_auto_kernel).
    Returns {p: {"kernel": KERNEL_SWEEP | KERNEL_COLUMN, "sweep_ms": ..,
    "column_ms": ..}}; results cached like tune()."""
    import torch

    from . import KERNEL_SWEEP, bk5_apply, bk5_matrices, bk5_set_auto_kernel, fill_uniform
    key = (f"{torch.cuda.get_device_name()}|apply|prec{prec}|layout{layout}|mass{int(bool(with_mass))}|"
           + ",".join(f"{p}:{min(int(E), max_elements)}" for p, E in sorted(orders)))
    cache = {}
    if use_cache and os.path.exists(CACHE):
        try:
            cache = json.load(open(CACHE))
        except (OSError, ValueError):
            cache = {}
    if key in cache:
        res = {int(p): v for p, v in cache[key].items()}
    else:
        dt = torch.float64 if prec == 0 else torch.float32
        res = {}
        for p, E in sorted(orders):
            E = max(1, min(int(E), max_elements))
            q = p + 1
            D = bk5_matrices(p)[0]
            u = fill_uniform(torch.empty(E * q ** 3, dtype=dt, device="cuda"), 3)
            G = fill_uniform(torch.empty(6 * E * q ** 3, dtype=dt, device="cuda"), 4, 0.5, 1.5)
            M = fill_uniform(torch.empty(E * q ** 3, dtype=dt, device="cuda"), 5, 0.5, 1.5) if with_mass else None
            v = torch.empty_like(u)
            t = {}
            for name, kern in (("sweep", KERNEL_SWEEP), ("column", KERNEL_COLUMN)):
                def run():
                    bk5_apply(p, E, D, G, u, v, prec=prec, layout=layout, mass=M, lam=1.0 if with_mass else 0.0,
                              kernel=kern)
                run()
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    run()
                e1.record()
                torch.cuda.synchronize()
                t[name] = e0.elapsed_time(e1) / reps
            res[p] = {"kernel": KERNEL_SWEEP if t["sweep"] <= t["column"] else KERNEL_COLUMN,
                      "sweep_ms": t["sweep"], "column_ms": t["column"]}
            del u, G, M, v
        if use_cache:
            cache[key] = {str(p): v for p, v in res.items()}
            try:
                os.makedirs(os.path.dirname(CACHE), exist_ok=True)
                json.dump(cache, open(CACHE, "w"), indent=1)
            except OSError:
                pass
    for p, r in res.items():
        bk5_set_auto_kernel(p, prec, layout, r["kernel"], with_mass=with_mass)
    if verbose:
        print("tune_apply: " + ", ".join(f"p={p}: {'sweep' if r['kernel'] == KERNEL_SWEEP else 'column'} "
                                         f"({r['sweep_ms']:.3f} / {r['column_ms']:.3f} ms)"
                                         for p, r in sorted(res.items())))
    return res
