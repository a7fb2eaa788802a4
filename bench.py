"""Benchmark of the GB300 bake-off operator apply.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (the headline configuration): BK5 collocated Laplacian, plain FP64,
p = 7 (P = Q = 8 GLL points), E = 262144 elements = 134,217,728 DoFs on a
64^3 grid of spacing h = 1/64 whose vertices are jittered by U[-0.15h, 0.15h]
(seeded), G = w detJ J^-1 J^-T with 6 symmetric factors generated directly in
the column layout G(e, f, k, i, j) (the layout of the reference's column-sweep
variants; BK5.cpp's interleaved layout is --layout 1), D the 8 x 8 GLL
derivative, u ~ U[-1, 1] (seeded).  All
inputs are synthetic (the reference names no dataset); the inputs (8.6 GB per
apply) are 65x the 129 MB L2, so no flush is needed between steps.

One step = one apply v = D^T G D u.  `value` is GDoF/s with u, G, v resident
in HBM (CUDA events on the launching stream, K steps); `e2e` is the same
apply through the C ABI from pinned host memory: every step copies u to the
device and v back (G, the operator, stays resident, as the reference's
`omp target data` region keeps it mapped, openmp/BK5.cpp:133).  The plain FP64
form uses the float-float engine (FP64 storage, FP64-accurate arithmetic on
the FP32 pipes: the GB300's FP64 pipe runs at 1/64 rate); the native-DFMA
engine and the FP32-storage mixed form are timed beside it ("forms").

`--impl reference` times the reference's algorithm on the host cores: the
oracle's C restatement of bk::SumFactorization<double, 8> (openmp/BK5.cpp:
19-103) with OpenMP over all cores, on a bounded sample of the same workload.
Multi-GPU (torchrun): replicas only (the apply has no exchange step); every
rank applies the operator to its own elements, value = all DoFs / max time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "GDOF/s per apply on 1 GB300: plain FP64 vs mixed/batched at stated error"
UNIT = "GDoF/s"
P_ORDER = 7
NX = 64
E_FULL = NX ** 3
SEED_U, SEED_G = 1, 2
H = 1.0 / NX
JITTER = 0.15


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--elements", type=int, default=None,
                    help="override E (profiling a smaller case); helmholtz: E_p = 2^(8-p) * elements / 64")
    ap.add_argument("--engine", default="ff", choices=["ff", "dfma"])
    ap.add_argument("--prec", default="fp64", choices=["fp64", "mixed", "fp32"],
                    help="form timed in the main loop (profiling; the headline is fp64)")
    ap.add_argument("--kernel", default="auto", choices=["auto", "sweep", "column"])
    ap.add_argument("--layout", type=int, default=2, help="G layout (0 factor, 1 interleaved, 2 column)")
    ap.add_argument("--no-forms", action="store_true", help="skip the side-by-side forms")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", default="bk5", choices=["bk5", "bk1", "bk3", "adjoint", "helmholtz"],
                    help="bk5: the headline; the others: the remaining configurations, one JSON line each")
    return ap.parse_args()


# ---- distributed plumbing -------------------------------------------------------

def dist_setup(n, backend="nccl"):
    """Rank, world size and local rank from the torchrun environment; the
    process group (NCCL between GPUs; gloo for the CPU tests) when world > 1.
    The apply has no exchange step: ranks only meet in the timing barrier and
    the max-over-ranks reduction (replicas)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        if not dist.is_initialized():
            dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    """The largest of the ranks' values (the slowest rank's time)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---- clocks -----------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- workload -----------------------------------------------------------------------

def make_inputs(bk, E, torch, layout=1):
    """Device inputs of the headline workload (FP64), built on the GPU."""
    D, x, w = bk.bk5_matrices(P_ORDER)
    Q = P_ORDER + 1
    n = E * Q ** 3
    u = torch.empty(n, dtype=torch.float64, device="cuda")
    G = torch.empty(6 * n, dtype=torch.float64, device="cuda")
    bk.fill_uniform(u, SEED_U, -1.0, 1.0)
    bk.geom_trilinear(Q, E, NX, NX, x, w, SEED_G, H, JITTER, G=G, layout=layout)
    torch.cuda.synchronize()
    return D, u, G


def time_loop(fn, steps, warmup, world, stream, torch):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(steps):
        fn()
    t1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    return t0.elapsed_time(t1) / 1e3 / steps   # seconds per step


def cpu_baseline_run(sample_E, steps, warmup=1, best=True):
    """The oracle's restatement of the reference's BK5 kernel in double, OpenMP
    over the host cores, on `sample_E` elements of the workload: `warmup`
    untimed applies, then `steps` timed ones; the rate from the best
    (bk::time_min, include/bk_common.h:182-192) or the mean time."""
    import numpy as np

    import oracle
    Q = P_ORDER + 1
    rng = np.random.default_rng(0)
    D = np.asarray(__import__("omp_bk_gb300").bk5_matrices(P_ORDER)[0])
    u = rng.uniform(-1, 1, sample_E * Q ** 3)
    G = rng.uniform(0.5, 1.5, sample_E * 6 * Q ** 3)
    oracle.lib(fast=True)
    for _ in range(warmup):
        oracle.bk5(Q, sample_E, D, G, u, fast=True)
    times = []
    for _ in range(steps):
        t = time.perf_counter()
        oracle.bk5(Q, sample_E, D, G, u, fast=True)
        times.append(time.perf_counter() - t)
    sec = min(times) if best else sum(times) / len(times)
    cores = os.cpu_count()
    how = f"min of {steps} applies" if best else f"mean of {steps} applies after {warmup} warm-up"
    return {"value": sample_E * Q ** 3 / sec / 1e9, "unit": UNIT, "cores": cores, "kind": "port",
            "ms_per_step": sec * 1e3,
            "sample": f"BK5 p=7 FP64, {sample_E} of the {E_FULL} elements (random u, G), {how}, "
                      f"OMP over {cores} host threads (oracle/bk_oracle.c, -O3)"}


def traffic_from_profiles():
    """DRAM bytes per launch of the headline kernel from the committed ncu
    summary (profiles/bk5_p7_fp64.json), scaled to the full workload."""
    path = os.path.join(ROOT, "profiles", "bk5_p7_fp64.json")
    try:
        d = json.load(open(path))
        return d.get("dram_bytes_per_launch_full")
    except (OSError, ValueError):
        return None


def measured_peak():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def run_reference(args):
    """The reference arm: the reference's BK5 p=7 FP64 kernel restated in C
    (the oracle port; the reference's own build is CMake-only and does not
    travel to the Arm machine) on the host cores, each step one apply of a
    32768-element sample of the workload, `--warmup` untimed steps first."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    steps, warmup = max(1, args.steps), max(0, args.warmup)
    cb = cpu_baseline_run(32768, steps, warmup, best=False)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": steps, "warmup": warmup, "ms_per_step": cb["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "BK5 p=7 FP64 apply, E=262144 (134M DoFs), CPU sample of 32768 elements",
                       "p": P_ORDER, "elements": E_FULL},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---- the other configurations ------------------------------------------------

def _events_ms(fn, steps, warmup, torch, graph=False):
    """Mean ms per call over `steps` calls after `warmup`, CUDA events on the
    current stream.  graph: the steps are captured once into a CUDA graph
    and replayed (the applies allocate and synchronize nothing), so that a
    launch of a few microseconds is not timed behind the host's per-call
    overhead."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    if graph:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for _ in range(steps):
                fn()
        g.replay()   # one untimed replay
        torch.cuda.synchronize()
        t0.record()
        g.replay()
        t1.record()
    else:
        t0.record()
        for _ in range(steps):
            fn()
        t1.record()
    torch.cuda.synchronize()
    return t0.elapsed_time(t1) / steps


def _rel(a, ref):
    d = (a.double() - ref).abs()
    return float(d.max() / ref.abs().max()), float(d.pow(2).mean().sqrt() / ref.pow(2).mean().sqrt())


def _line(args, workload, value, ms, dtype, extra):
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
           "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": dtype, "data": "synthetic", "config": {"workload": workload}}
    out.update(extra)
    print(json.dumps(out), flush=True)


def run_bk1(args):
    """BK1 mass apply p = 3 (P = 4 GLL nodes, Q = 5 Gauss points), E = 4096,
    affine elements (h = 1/16, U[-0.2, 0.2] perturbation), u ~ U[-1, 1]."""
    import torch

    import omp_bk_gb300 as bk
    p, E = 3, args.elements or 4096
    P, Q = p + 1, p + 2
    B, _, xq, wq, _ = bk.bk1_bk3_matrices(p)
    qd = torch.empty(E * Q ** 3, dtype=torch.float64, device="cuda")
    bk.geom_affine(Q, E, xq, wq, 21, 1.0 / 16, 0.2, qdata=qd)
    u = bk.fill_uniform(torch.empty(E * P ** 3, dtype=torch.float64, device="cuda"), 22)
    v = torch.empty_like(u)
    dofs = E * P ** 3
    steps, warm = max(args.steps, 20), max(args.warmup, 3)
    # one apply is ~15 us: the applies are timed as one CUDA graph of `steps`
    # launches (device time; a host-timed loop measured the ctypes call)
    ms = _events_ms(lambda: bk.bk1_apply(p, E, B, qd, u, v), steps, warm, torch, graph=True)
    forms = {}
    ref = v.clone()
    vd = torch.empty_like(v)
    md = _events_ms(lambda: bk.bk1_apply(p, E, B, qd, u, vd, engine=bk.ENGINE_DFMA), steps, warm, torch, graph=True)
    forms["fp64_dfma"] = {"gdofs": dofs / md / 1e6, "rel_max_err": _rel(vd, ref)[0]}
    u32, q32 = u.float(), qd.float()
    v32 = torch.empty_like(u32)
    for name, pr in (("fp32", bk.PREC_FP32), ("mixed", bk.PREC_MIXED)):
        m32 = _events_ms(lambda: bk.bk1_apply(p, E, B, q32, u32, v32, prec=pr), steps, warm, torch, graph=True)
        forms[name] = {"gdofs": dofs / m32 / 1e6, "rel_max_err": _rel(v32, ref)[0]}
    import oracle
    t = time.perf_counter()
    host = oracle.bk1(Q, E, B, qd.cpu().numpy(), u.cpu().numpy(), fast=True)
    cpu_s = time.perf_counter() - t
    err = float(abs(torch.from_numpy(host) - ref.cpu()).max() / ref.abs().max())
    _line(args, f"BK1 mass apply p={p} (P=4 GLL, Q=5 Gauss), E={E}, FP64 float-float, L2-resident (8.3 MB), "
                f"timed as one CUDA graph of {steps} applies",
          dofs / ms / 1e6, ms, "f64",
          {"forms": forms, "rel_max_err_vs_oracle": err,
           "cpu_baseline": {"value": dofs / cpu_s / 1e9, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                            "sample": f"full workload, one apply (oracle/bk_oracle.c, OpenMP)"}})


def run_bk3(args):
    """BK3 p = 6 (P = 7, Q = 8), E = 131072, affine elements: FP64 against the
    mixed form, max and RMS relative error for u ~ U[-1,1] and the smooth
    u = sin(pi x) sin(pi y) sin(pi z) at the GLL nodes."""
    import torch

    import omp_bk_gb300 as bk
    p, E = 6, args.elements or 131072
    P, Q = p + 1, p + 2
    B, D, xq, wq, xn = bk.bk1_bk3_matrices(p)
    G = torch.empty(E * 6 * Q ** 3, dtype=torch.float64, device="cuda")
    bk.geom_affine(Q, E, xq, wq, 31, 1.0 / 64, 0.2, G=G, layout=bk.LAYOUT_FACTOR)
    u_rand = bk.fill_uniform(torch.empty(E * P ** 3, dtype=torch.float64, device="cuda"), 32)
    X = torch.empty(E * P ** 3 * 3, dtype=torch.float64, device="cuda")
    bk.coords_affine(P, E, 64, 64, xn, 31, 1.0 / 64, 0.2, X)
    X = X.view(-1, 3)
    u_smooth = (torch.sin(math.pi * X[:, 0]) * torch.sin(math.pi * X[:, 1]) * torch.sin(math.pi * X[:, 2])).contiguous()
    dofs = E * P ** 3
    steps, warm = max(args.steps // 4, 10), max(args.warmup, 3)
    v = torch.empty_like(u_rand)
    ms = _events_ms(lambda: bk.bk3_apply(p, E, B, D, G, u_rand, v), steps, warm, torch)
    G32 = G.float()
    v32 = torch.empty(E * P ** 3, dtype=torch.float32, device="cuda")
    errs = {}
    G32d = G32.double()
    vr = torch.empty_like(v)
    for name, uu in (("random", u_rand), ("smooth", u_smooth)):
        bk.bk3_apply(p, E, B, D, G, uu, v)
        u32 = uu.float()
        bk.bk3_apply(p, E, B, D, G32, u32, v32, prec=bk.PREC_MIXED)
        mx, rms = _rel(v32, v)
        # the same split for FP64 applied to the FP32-rounded inputs: the
        # part of the error that storing u and G in FP32 causes by itself
        # (large for smooth u, whose image cancels) and the part the FP32
        # arithmetic adds
        bk.bk3_apply(p, E, B, D, G32d, u32.double(), vr)
        mx_in, rms_in = _rel(vr, v)
        mx_ar, rms_ar = _rel(v32, vr)
        errs[name] = {"rel_max": mx, "rel_rms": rms, "input_rounding_rel_max": mx_in,
                      "input_rounding_rel_rms": rms_in, "arithmetic_rel_max": mx_ar, "arithmetic_rel_rms": rms_ar}
    mm = _events_ms(lambda: bk.bk3_apply(p, E, B, D, G32, u32, v32, prec=bk.PREC_MIXED), steps, warm, torch)
    vd = torch.empty_like(v)
    md = _events_ms(lambda: bk.bk3_apply(p, E, B, D, G, u_smooth, vd, engine=bk.ENGINE_DFMA), max(3, steps // 4),
                    2, torch)
    # G split once into float-float pairs (bk_g_to_ff, outside the timed region)
    Gff = bk.g_to_ff(G)
    mg = _events_ms(lambda: bk.bk3_apply(p, E, B, D, Gff, u_rand, vd, gform=bk.G_FF), steps, warm, torch)
    bk.bk3_apply(p, E, B, D, G, u_rand, v)
    split_diff = float((vd - v).abs().max())
    del Gff
    bytes64 = 8 * (2 * dofs + 6 * E * Q ** 3)
    _line(args, f"BK3 Poisson p={p} (P=7 GLL, Q=8 Gauss), E={E}, FP64 float-float vs mixed (FP32 storage)",
          dofs / ms / 1e6, ms, "f64",
          {"forms": {"fp64_ff": {"gdofs": dofs / ms / 1e6, "hbm_frac": bytes64 / ms / 1e6 / measured_peak()[0]},
                     "fp64_dfma": {"gdofs": dofs / md / 1e6},
                     "fp64_ff_split_g": {"gdofs": dofs / mg / 1e6, "max_abs_diff_vs_fp64_ff": split_diff,
                                         "hbm_frac": bytes64 / mg / 1e6 / measured_peak()[0]},
                     "mixed": {"gdofs": dofs / mm / 1e6, "speedup_vs_fp64": ms / mm,
                               "hbm_frac": bytes64 / 2 / mm / 1e6 / measured_peak()[0], "errors": errs}}})


def run_adjoint(args):
    """BK3 adjoint p = 4 (P = 5, Q = 6), E = 65536, log k ~ N(0, 0.5^2):
    forward + backward timing and the central-difference check (h = 1e-6)."""
    import torch

    import omp_bk_gb300 as bk
    p, E = 4, args.elements or 65536
    P, Q = p + 1, p + 2
    B, D, xq, wq, _ = bk.bk1_bk3_matrices(p)
    G = torch.empty(E * 6 * Q ** 3, dtype=torch.float64, device="cuda")
    bk.geom_affine(Q, E, xq, wq, 41, 1.0 / 16, 0.2, G=G, layout=bk.LAYOUT_FACTOR)
    k = bk.fill_lognormal(torch.empty(E * Q ** 3, dtype=torch.float64, device="cuda"), 42, 0.5)
    u = bk.fill_uniform(torch.empty(E * P ** 3, dtype=torch.float64, device="cuda"), 43)
    f = bk.fill_uniform(torch.empty(E * P ** 3, dtype=torch.float64, device="cuda"), 44)
    r = torch.empty_like(u)
    dk = torch.empty_like(k)
    dG = torch.empty_like(G)

    def fwd(kk, GG, rr, eng=bk.ENGINE_AUTO):
        bk.bk3_apply(p, E, B, D, GG, u, rr, k=kk, engine=eng)
        bk.axpby(-1.0, f, 1.0, rr)

    steps, warm = max(args.steps // 4, 10), max(args.warmup, 3)
    mf = _events_ms(lambda: fwd(k, G, r), steps, warm, torch)
    mb = _events_ms(lambda: bk.bk3_adjoint(p, E, B, D, G, k, u, r, dk, dG), steps, warm, torch)
    # the backward on G split once into float-float pairs (bitwise the same
    # gradients)
    Gff = bk.g_to_ff(G)
    dk2, dG2 = torch.empty_like(dk), torch.empty_like(dG)
    mbg = _events_ms(lambda: bk.bk3_adjoint(p, E, B, D, Gff, k, u, r, dk2, dG2, gform=bk.G_FF), steps, warm, torch)
    bk.bk3_adjoint(p, E, B, D, G, k, u, r, dk, dG)
    split_same = bool(torch.equal(dk, dk2) and torch.equal(dG, dG2))
    del Gff, dk2, dG2
    ws = bk.dot_workspace(6 * E * Q ** 3)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    fwd(k, G, r, bk.ENGINE_DFMA)
    bk.bk3_adjoint(p, E, B, D, G, k, u, r, dk, dG)
    h = 1e-6
    worst = 0.0
    rp, rm = torch.empty_like(r), torch.empty_like(r)
    dkd, dGd = torch.empty_like(k), torch.empty_like(G)
    for t in range(64):
        bk.fill_uniform(dkd, 1000 + t)
        bk.fill_uniform(dGd, 2000 + t)
        dGd.mul_(G.abs().mean())
        fwd(k + h * dkd, G + h * dGd, rp, bk.ENGINE_DFMA)
        fwd(k - h * dkd, G - h * dGd, rm, bk.ENGINE_DFMA)
        bk.dot(rp - rm, rp + rm, out, ws)
        fd = out.item() / (4 * h)
        bk.dot(dk, dkd, out, ws)
        an = out.item()
        bk.dot(dG, dGd, out, ws)
        an += out.item()
        worst = max(worst, abs(fd - an) / abs(an))
    qdofs = E * Q ** 3
    _line(args, f"BK3 adjoint p={p} (P=5, Q=6), E={E}, FP64: dL/dk, dL/dG of 1/2|A(k)u - f|^2",
          qdofs / mb / 1e6, mb, "f64",
          {"adjoint": {"backward_ms": mb, "forward_ms": mf, "backward_gpoints_s": qdofs / mb / 1e6,
                       "backward_hbm_gbs": 8 * (2 * E * P ** 3 + 14 * qdofs) / mb / 1e6,
                       "backward_split_g_gpoints_s": qdofs / mbg / 1e6, "split_g_bitwise": split_same,
                       "fd_directions": 64, "fd_step": h, "fd_max_rel_err": worst},
           "unit_note": "value = quadrature points per second of the backward kernel (G points/s)"})


def run_helmholtz(args):
    """Mixed-order Helmholtz (BK5 + GLL mass, lambda = 1), p = 2..8, E_p =
    2^(8-p) 4096: tiles tuned per order, one persistent launch, CG to 1e-10
    with FP32 inner applies and FP64 refinement; against per-order FP64
    launches."""
    import torch

    import omp_bk_gb300 as bk
    from omp_bk_gb300 import helmholtz as hz
    from omp_bk_gb300 import tune
    orders = hz.config_orders()
    if args.elements:
        orders = [(p, max(1, (2 ** (8 - p)) * args.elements // 64)) for p, _ in orders]
    best = tune.tune(orders)
    plan = hz.HelmholtzPlan([(p, E, best[p]) for p, E in orders])
    G, M = plan.geometry(seed=11)
    G32, M32 = G.float(), M.float()
    ustar = bk.fill_uniform(torch.empty(plan.n, dtype=torch.float64, device="cuda"), 5)
    f = torch.empty_like(ustar)
    plan.apply(G, M, 1.0, ustar, f, prec=bk.PREC_FP64)
    u32, v32, v64 = ustar.float(), torch.empty(plan.n, dtype=torch.float32, device="cuda"), torch.empty_like(ustar)
    steps, warm = max(args.steps // 4, 10), max(args.warmup, 3)
    # every apply below is timed as one CUDA graph of its launches (device
    # time: the seven per-order launches of a Python loop would otherwise be
    # timed behind the host)
    m_multi = _events_ms(lambda: plan.apply(G32, M32, 1.0, u32, v32, prec=bk.PREC_MIXED), steps, warm, torch,
                         graph=True)
    m_multi64 = _events_ms(lambda: plan.apply(G, M, 1.0, ustar, v64, prec=bk.PREC_FP64), max(3, steps // 4), 2,
                           torch, graph=True)
    Dp = {p: bk.bk5_matrices(p)[0] for p in plan.p}

    def per_order(prec, GG, MM, uu, vv):
        for kk, p in enumerate(plan.p):
            q, E = p + 1, plan.E[kk]
            su = slice(plan.uoff[kk], plan.uoff[kk] + E * q ** 3)
            sg = slice(plan.goff[kk], plan.goff[kk] + 6 * E * q ** 3)
            bk.bk5_apply(p, E, Dp[p], GG[sg], uu[su], vv[su], prec=prec, layout=bk.LAYOUT_COLUMN, mass=MM[su],
                         lam=1.0)

    aligned = all((o * 8) % 16 == 0 for o in plan.uoff) and all((o * 8) % 16 == 0 for o in plan.goff)
    m_per64 = _events_ms(lambda: per_order(bk.PREC_FP64, G, M, ustar, v64), max(3, steps // 4), 2, torch,
                         graph=True) if aligned else None
    aligned32 = all((o * 4) % 16 == 0 for o in plan.uoff) and all((o * 4) % 16 == 0 for o in plan.goff)
    m_per32 = _events_ms(lambda: per_order(bk.PREC_MIXED, G32, M32, u32, v32), steps, warm, torch, graph=True) \
        if aligned32 else None
    # the column body of the same launch (tiles tuned for it)
    best_col = tune.tune(orders, kernel=bk.KERNEL_COLUMN)
    plan_col = hz.HelmholtzPlan([(p, E, best_col[p]) for p, E in orders])
    plan_col.set_kernel(bk.KERNEL_COLUMN)
    m_col = _events_ms(lambda: plan_col.apply(G32, M32, 1.0, u32, v32, prec=bk.PREC_MIXED), steps, warm, torch,
                       graph=True)
    plan_col.close()
    x = torch.zeros_like(ustar)
    plan.cg(G, M, G32, M32, 1.0, f, x, rtol=1e-10, allow_noconv=True)   # builds the graph
    x.zero_()
    torch.cuda.synchronize()
    t = time.perf_counter()
    st = plan.cg(G, M, G32, M32, 1.0, f, x, rtol=1e-10, allow_noconv=True)
    torch.cuda.synchronize()
    solve_s = time.perf_counter() - t
    err = float(torch.linalg.norm(x - ustar) / torch.linalg.norm(ustar))
    _line(args, f"mixed-order Helmholtz p=2..8, E_p=2^(8-p)*{orders[-1][1]} ({plan.n} DoFs), one persistent launch",
          plan.n / m_multi / 1e6, m_multi, "f32",
          {"helmholtz": {"dofs": plan.n, "tiles": plan.ntiles, "tile_elems": best,
                         "kernel": {bk.KERNEL_SWEEP: "sweep (even-odd)", bk.KERNEL_COLUMN: "column"}[plan.kernel],
                         "multi_mixed_gdofs": plan.n / m_multi / 1e6, "multi_fp64_gdofs": plan.n / m_multi64 / 1e6,
                         "multi_mixed_column_gdofs": plan.n / m_col / 1e6, "tile_elems_column": best_col,
                         "per_order_mixed_gdofs": (plan.n / m_per32 / 1e6) if m_per32 else None,
                         "per_order_fp64_gdofs": (plan.n / m_per64 / 1e6) if m_per64 else None,
                         "cg": st, "cg_seconds": solve_s, "solution_rel_err": err}})


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "bk5":
        {"bk1": run_bk1, "bk3": run_bk3, "adjoint": run_adjoint, "helmholtz": run_helmholtz}[args.workload](args)
        return 0
    import torch

    import omp_bk_gb300 as bk
    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    E = args.elements or E_FULL
    Q = P_ORDER + 1
    dofs = E * Q ** 3
    D, u, G = make_inputs(bk, E, torch, args.layout)
    v = torch.empty_like(u)
    engine = bk.ENGINE_FF if args.engine == "ff" else bk.ENGINE_DFMA
    kernel = {"auto": bk.KERNEL_AUTO, "sweep": bk.KERNEL_SWEEP, "column": bk.KERNEL_COLUMN}[args.kernel]
    prec = {"fp64": bk.PREC_FP64, "mixed": bk.PREC_MIXED, "fp32": bk.PREC_FP32}[args.prec]
    if prec != bk.PREC_FP64:
        u, G = u.float(), G.float()
        v = torch.empty_like(u)
    kw = dict(engine=engine, layout=args.layout, kernel=kernel, stream=stream)

    def apply():
        bk.bk5_apply(P_ORDER, E, D, G, u, v, prec=prec, **kw)

    steps, warmup = args.steps, max(args.warmup, 3)
    with ClockSampler(local) as clk:
        t = time_loop(apply, steps, warmup, world, stream, torch)
    t = max_over_ranks(t, world)
    value = world * dofs / t / 1e9
    bytes_per_apply = u.element_size() * (2 + 6) * dofs
    peak, peak_kind = measured_peak()
    achieved = bytes_per_apply / t / 1e9
    traffic = traffic_from_profiles() if E == E_FULL else None

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": warmup,
           "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64" if prec == bk.PREC_FP64 else "f32", "data": "synthetic",
           "config": {"workload": f"BK5 collocated Laplacian p={P_ORDER} (P=Q=8 GLL) FP64 apply, E={E} "
                                  f"({dofs} DoFs), jittered trilinear mesh, G6 layout {args.layout}",
                      "p": P_ORDER, "elements": E, "engine": args.engine, "prec": args.prec, "kernel": args.kernel,
                      "layout": args.layout, "l2": "inputs 8.6 GB >> 129 MB L2, no flush",
                      "parallelism": f"replicas x{world}"},
           "gpu_launches": steps,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "traffic": traffic,
                        "note": f"peak = {peak_kind} copy bandwidth (MEASURED_PEAKS.json hbm_gbs); algorithmic "
                                f"bytes = 8 B x (u + v + 6 G) per DoF"},
           "clocks": clk.summary()}

    # end to end through the C ABI on HOST arrays (bk5_apply_host): pinned
    # host u -> device -> apply -> pinned host v every step, the elements cut
    # into 16 chunks whose copies in and out (two copy streams) overlap the
    # applies of the neighbouring chunks
    if not args.no_e2e:
        uh = torch.empty(u.numel(), dtype=u.dtype, pin_memory=True)
        vh = torch.empty_like(uh)
        uh.copy_(u)
        hp = bk.HostPlan(5, P_ORDER, E, prec=prec)

        def step_e2e():
            hp.apply(uh, vh, G=G, D=D, engine=engine, layout=args.layout, kernel=kernel, stream=stream)

        # three timed rounds, the best kept (the reference's time_min); the
        # host link is shared with the machine's other work, so the rounds
        # are reported too
        rounds = [max_over_ranks(time_loop(step_e2e, max(3, steps // 10), 2, world, stream, torch), world)
                  for _ in range(3)]
        te = min(rounds)
        torch.cuda.synchronize()
        e2e_err = float((vh.to(v.device) - v).abs().max())
        hp.close()
        out["e2e"] = {"value": world * dofs / te / 1e9, "unit": UNIT, "h2d_bytes_per_step": u.element_size() * dofs,
                      "d2h_bytes_per_step": u.element_size() * dofs, "ms_per_step": te * 1e3,
                      "rounds_ms_per_step": [r * 1e3 for r in rounds],
                      "max_abs_diff_vs_device_apply": e2e_err,
                      "note": "bk5_apply_host: G (6.4 GB) resident on the device; u in, v out every step "
                              "from/to pinned host memory in 16 element chunks, copies overlapping the applies"}

    # the forms side by side, with their error against the FP64 result
    if not args.no_forms and rank == 0 and prec == bk.PREC_FP64:
        forms = {}
        ref = v.clone()
        forms["fp64_ff"] = {"gdofs": value / world, "rel_err_vs_fp64": 0.0}
        vd = torch.empty_like(v)
        td = time_loop(lambda: bk.bk5_apply(P_ORDER, E, D, G, u, vd, engine=bk.ENGINE_DFMA, layout=args.layout,
                                            stream=stream),
                       max(3, steps // 20), 2, 1, stream, torch)
        forms["fp64_dfma"] = {"gdofs": dofs / td / 1e9,
                              "rel_err_vs_fp64": float((vd - ref).abs().max() / ref.abs().max())}
        # G split once into float-float pairs (bk_g_to_ff, outside the timed
        # region, like the relayout of G): the same bytes, no split per load
        if args.engine == "ff":
            Gff = bk.g_to_ff(G)
            tg = time_loop(lambda: bk.bk5_apply(P_ORDER, E, D, Gff, u, vd, engine=engine, layout=args.layout,
                                                gform=bk.G_FF, stream=stream),
                           max(3, steps // 4), 3, 1, stream, torch)
            forms["fp64_ff_split_g"] = {"gdofs": dofs / tg / 1e9,
                                        "max_abs_diff_vs_fp64_ff": float((vd - ref).abs().max()),
                                        "hbm_frac": 8 * 8 * dofs / tg / 1e9 / peak}
            del Gff
        del vd
        u32, G32 = u.float(), G.float()
        v32 = torch.empty_like(u32)
        for name, prec in (("mixed_fp32_storage", bk.PREC_MIXED), ("fp32", bk.PREC_FP32)):
            tm = time_loop(lambda: bk.bk5_apply(P_ORDER, E, D, G32, u32, v32, prec=prec, layout=args.layout,
                                                stream=stream),
                           max(3, steps // 4), 3, 1, stream, torch)
            err = float((v32.double() - ref).abs().max() / ref.abs().max())
            forms[name] = {"gdofs": dofs / tm / 1e9, "rel_err_vs_fp64": err,
                           "hbm_frac": 4 * 8 * dofs / tm / 1e9 / peak}
        out["forms"] = forms
        del u32, G32, v32

    if rank == 0 and world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline_run(32768, 3)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
