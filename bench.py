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

The headline's own result is checked against the FP64 oracle (the first and
the last 1024 elements of u and G copied to the host, oracle.bk5): `parity`.
The default run also measures the other four configurations and puts them
under `configs` (BK1 p=3, BK3 p=6 FP64 and mixed with both inputs, the BK3
adjoint p=4, the mixed-order Helmholtz launch and CG), each with its error
against the oracle and its own CPU baseline; `--workload X` prints one of
them alone.

`--impl reference` times the reference's algorithm on the host cores: the
oracle's C restatement of bk::SumFactorization<double, 8> (openmp/BK5.cpp:
19-103), pinned to the reference's own kernels, with OpenMP over all cores,
on the whole workload (E = 262144) built on the host by the oracle's
restatement of the same seeded generators, G in BK5.cpp's interleaved layout.
It imports nothing of the GPU package.  Both arms report the mean time per
step over K steps after W warm-up steps.
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
    ap.add_argument("--no-configs", action="store_true", help="skip the other four configurations")
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


def headline_config(E):
    """The workload both arms report (the same dict in both lines)."""
    return {"workload": f"BK5 collocated Laplacian p={P_ORDER} (P=Q=8 GLL) FP64 apply, E={E} "
                        f"({E * (P_ORDER + 1) ** 3} DoFs), jittered trilinear mesh (h=1/{NX}, jitter {JITTER}h), "
                        f"u ~ U[-1,1]", "p": P_ORDER, "elements": E}


def host_inputs(E):
    """The headline's inputs built on the host by the oracle (no GPU code):
    D (8 x 8 GLL derivative), u ~ U[-1,1] (seed SEED_U), G (seed SEED_G) in
    BK5.cpp's interleaved layout G(e, i, j, f, k)."""
    import oracle
    Q = P_ORDER + 1
    D, x, w = oracle.bk5_matrices(P_ORDER)
    u = oracle.uniform(E * Q ** 3, SEED_U, -1.0, 1.0, fast=True)
    G, _, _ = oracle.geom_trilinear(Q, 0, E, NX, NX, x, w, SEED_G, H, JITTER, layout=1, fast=True)
    return D, u, G


def cpu_bk5_run(E, steps, warmup):
    """The oracle's restatement of the reference's BK5 kernel
    (bk::SumFactorization<double, 8>, openmp/BK5.cpp:19-103) in double, OpenMP
    over all host cores, on the whole workload: `warmup` untimed applies, then
    `steps` timed ones; the rate from the mean time per apply (the GPU arm's
    statistic)."""
    import oracle
    Q = P_ORDER + 1
    t = time.perf_counter()
    D, u, G = host_inputs(E)
    gen_s = time.perf_counter() - t
    oracle.lib(fast=True)
    out = None
    for _ in range(warmup):
        out = oracle.bk5(Q, E, D, G, u, fast=True)
    t = time.perf_counter()
    for _ in range(steps):
        out = oracle.bk5(Q, E, D, G, u, fast=True)
    sec = (time.perf_counter() - t) / steps
    cores = os.cpu_count()
    return {"value": E * Q ** 3 / sec / 1e9, "unit": UNIT, "cores": cores, "kind": "port",
            "ms_per_step": sec * 1e3, "input_build_s": gen_s,
            "output_norm": float(__import__("numpy").linalg.norm(out)),
            "sample": f"the whole workload (E={E}), mean of {steps} applies after {warmup} warm-up, OpenMP over "
                      f"{cores} host threads: oracle/bk_oracle.c (-O3), the restatement of bk::SumFactorization"
                      f"<double, 8> pinned to the reference's own kernels; inputs from oracle/bk_geom_oracle.c "
                      f"(the same seeded generators as the GPU's)"}


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
    travel to the Arm machine) on the host cores, each step one apply of the
    whole workload, `--warmup` untimed steps first.  Rank 0 alone runs it."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    steps, warmup = max(1, args.steps), max(0, args.warmup)
    E = args.elements or E_FULL
    cb = cpu_bk5_run(E, steps, warmup)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": steps, "warmup": warmup, "ms_per_step": cb["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": headline_config(E), "cpu_baseline": cb,
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


def _hostrel(a, ref):
    """max |a - ref| / max |ref| of two host arrays (the harness's rel-max,
    include/bk_harness.h:74-83)."""
    import numpy as np
    a, ref = np.asarray(a, dtype=np.float64).ravel(), np.asarray(ref, dtype=np.float64).ravel()
    return float(np.abs(a - ref).max() / np.abs(ref).max())


def _cpu_time(fn, steps=3):
    """Mean seconds of `steps` calls of a host function after one warm-up."""
    fn()
    t = time.perf_counter()
    for _ in range(steps):
        fn()
    return (time.perf_counter() - t) / steps


def _cpu_line(units, sec, what):
    return {"value": units / sec / 1e9, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "ms_per_step": sec * 1e3, "sample": what}


def run_bk1(args):
    """BK1 mass apply p = 3 (P = 4 GLL nodes, Q = 5 Gauss points), E = 4096,
    affine elements (h = 1/16, U[-0.2, 0.2] perturbation), u ~ U[-1, 1]."""
    import torch

    import omp_bk_gb300 as bk
    import oracle
    p, E = 3, args.elements or 4096
    P, Q = p + 1, p + 2
    B, _, xq, wq, _ = bk.bk1_bk3_matrices(p)
    qd = torch.empty(E * Q ** 3, dtype=torch.float64, device="cuda")
    bk.geom_affine(Q, E, xq, wq, 21, 1.0 / 16, 0.2, qdata=qd)
    u = bk.fill_uniform(torch.empty(E * P ** 3, dtype=torch.float64, device="cuda"), 22)
    v = torch.empty_like(u)
    dofs = E * P ** 3
    steps, warm = max(args.steps, 20), max(args.warmup, 3)
    # one apply is ~10 us: the applies are timed as one CUDA graph of `steps`
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
        forms[name] = {"gdofs": dofs / m32 / 1e6, "rel_max_err": _rel(v32, ref)[0],
                       "hbm_frac_if_from_hbm": 4 * (2 * dofs + E * Q ** 3) / m32 / 1e6 / measured_peak()[0]}
    qh, uh = qd.cpu().numpy(), u.cpu().numpy()
    err = _hostrel(ref.cpu().numpy(), oracle.bk1(Q, E, B, qh, uh))
    sec = _cpu_time(lambda: oracle.bk1(Q, E, B, qh, uh, fast=True))
    return {"workload": f"BK1 mass apply p={p} (P=4 GLL, Q=5 Gauss), E={E}, affine mesh, FP64 float-float, "
                        f"L2-resident (8.3 MB), timed as one CUDA graph of {steps} applies",
            "gdofs": dofs / ms / 1e6, "ms_per_apply": ms, "dtype": "f64",
            "bytes_per_apply": 8 * (2 * dofs + E * Q ** 3),
            "l2_frac_note": "8.3 MB per apply stays in the 129 MB L2: no HBM roofline applies",
            "rel_max_err_vs_oracle": err, "oracle_elements": E, "forms": forms,
            "cpu_baseline": _cpu_line(dofs, sec, f"the whole workload, mean of 3 applies, oracle/bk_oracle.c "
                                                 f"(-O3, OpenMP)")}


def run_bk3(args):
    """BK3 p = 6 (P = 7, Q = 8), E = 131072, affine elements: FP64 against the
    mixed form, max and RMS relative error for u ~ U[-1,1] and the smooth
    u = sin(pi x) sin(pi y) sin(pi z) at the GLL nodes."""
    import torch

    import omp_bk_gb300 as bk
    import oracle
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
    del X
    dofs = E * P ** 3
    steps, warm = max(args.steps // 4, 10), max(args.warmup, 3)
    v = torch.empty_like(u_rand)
    ms = _events_ms(lambda: bk.bk3_apply(p, E, B, D, G, u_rand, v), steps, warm, torch)
    # the FP64 result against the oracle on its first elements
    ns = min(E, 512)
    Gh, uh = G[: ns * 6 * Q ** 3].cpu().numpy(), u_rand[: ns * P ** 3].cpu().numpy()
    err64 = _hostrel(v[: ns * P ** 3].cpu().numpy(), oracle.bk3(Q, ns, B, D, Gh, uh))
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
        errs[name] = {"rel_max": mx, "rel_rms": rms, "meets_1e-6": mx <= 1e-6,
                      "input_rounding_rel_max": mx_in, "input_rounding_rel_rms": rms_in,
                      "arithmetic_rel_max": mx_ar, "arithmetic_rel_rms": rms_ar}
    del G32d, vr
    errs["note"] = ("smooth u: storing u and G in FP32 alone gives input_rounding_rel_max (the operator's image of "
                    "a smooth field cancels), so no FP32-storage form can meet 1e-6 there; the FP64 forms and the "
                    "CG with FP64 refinement (Helmholtz, 1e-10) do")
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
    peak = measured_peak()[0]
    bytes64 = 8 * (2 * dofs + 6 * E * Q ** 3)
    nc = min(E, 8192)
    Gc, uc = G[: nc * 6 * Q ** 3].cpu().numpy(), u_rand[: nc * P ** 3].cpu().numpy()
    sec = _cpu_time(lambda: oracle.bk3(Q, nc, B, D, Gc, uc, fast=True))
    return {"workload": f"BK3 Poisson p={p} (P=7 GLL, Q=8 Gauss), E={E}, affine mesh, FP64 float-float vs mixed "
                        f"(FP32 storage)",
            "gdofs": dofs / ms / 1e6, "ms_per_apply": ms, "dtype": "f64", "hbm_frac": bytes64 / ms / 1e6 / peak,
            "rel_max_err_vs_oracle": err64, "oracle_elements": ns,
            "forms": {"fp64_ff": {"gdofs": dofs / ms / 1e6, "hbm_frac": bytes64 / ms / 1e6 / peak},
                      "fp64_dfma": {"gdofs": dofs / md / 1e6},
                      "fp64_ff_split_g": {"gdofs": dofs / mg / 1e6, "max_abs_diff_vs_fp64_ff": split_diff,
                                          "hbm_frac": bytes64 / mg / 1e6 / peak},
                      "mixed": {"gdofs": dofs / mm / 1e6, "speedup_vs_fp64": ms / mm,
                                "hbm_frac": bytes64 / 2 / mm / 1e6 / peak, "errors": errs}},
            "cpu_baseline": _cpu_line(nc * P ** 3, sec, f"{nc} of the {E} elements, mean of 3 applies, "
                                                        f"oracle/bk_oracle.c (-O3, OpenMP)")}


def run_adjoint(args):
    """BK3 adjoint p = 4 (P = 5, Q = 6), E = 65536, log k ~ N(0, 0.5^2):
    forward + backward timing, the FP64 host gradient of the oracle on the
    first elements and the central-difference check (h = 1e-6, 64
    directions)."""
    import torch

    import omp_bk_gb300 as bk
    import oracle
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
    # the FP64 host gradient on the first elements
    ns = min(E, 256)
    hs = lambda t, n: t[:n].cpu().numpy()   # noqa: E731
    args_h = (hs(G, ns * 6 * Q ** 3), hs(k, ns * Q ** 3), hs(u, ns * P ** 3), hs(r, ns * P ** 3))
    rdk, rdG = oracle.bk3_adjoint(Q, ns, B, D, *args_h)
    host_err = max(_hostrel(hs(dk, ns * Q ** 3), rdk), _hostrel(hs(dG, ns * 6 * Q ** 3), rdG))
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
    nc = min(E, 4096)
    args_c = (hs(G, nc * 6 * Q ** 3), hs(k, nc * Q ** 3), hs(u, nc * P ** 3), hs(r, nc * P ** 3))
    sec = _cpu_time(lambda: oracle.bk3_adjoint(Q, nc, B, D, *args_c))
    peak = measured_peak()[0]
    bwd_bytes = 8 * (2 * E * P ** 3 + 14 * qdofs)
    return {"workload": f"BK3 adjoint p={p} (P=5, Q=6), E={E}, FP64: dL/dk, dL/dG of 1/2|A(k)u - f|^2",
            "gpoints_s": qdofs / mb / 1e6, "unit_note": "G points/s: quadrature points per second of the backward",
            "backward_ms": mb, "forward_ms": mf, "dtype": "f64",
            "backward_hbm_gbs": bwd_bytes / mb / 1e6, "hbm_frac": bwd_bytes / mb / 1e6 / peak,
            "backward_split_g_gpoints_s": qdofs / mbg / 1e6, "split_g_bitwise": split_same,
            "rel_max_err_vs_oracle_gradient": host_err, "oracle_elements": ns,
            "fd_directions": 64, "fd_step": h, "fd_max_rel_err": worst,
            "cpu_baseline": _cpu_line(nc * Q ** 3, sec, f"G points/s of the oracle's host gradient on {nc} of the "
                                                        f"{E} elements, mean of 3 (oracle/bk_oracle.c, OpenMP)")}


def run_helmholtz(args):
    """Mixed-order Helmholtz (BK5 + GLL mass, lambda = 1), p = 2..8, E_p =
    2^(8-p) 4096: tiles tuned per order, one persistent launch, CG to 1e-10
    with FP32 inner applies and FP64 refinement; against per-order FP64
    launches."""
    import torch

    import omp_bk_gb300 as bk
    import oracle
    from omp_bk_gb300 import helmholtz as hz
    from omp_bk_gb300 import tune
    orders = hz.config_orders()
    if args.elements:
        orders = [(p, max(1, (2 ** (8 - p)) * args.elements // 64)) for p, _ in orders]
    # tuned on the configuration itself (no cap on the elements per order:
    # a full apply takes a third of a millisecond), so that the tiles fit
    # its balance of orders
    emax = max(E for _, E in orders)
    tuned = tune.tune(orders, max_elements=emax)
    # the FP64-storage launches (float-float: the solver's residual and the
    # FP64 persistent apply) tuned apart: their arithmetic and shared memory
    # per element differ from the FP32 forms'
    tuned64 = tune.tune(orders, prec=bk.PREC_FP64, max_elements=emax)
    plan = tune.make_plan(orders, tuned, fp64=tuned64)
    G, M = plan.geometry(seed=11)
    G32, M32 = G.float(), M.float()
    ustar = bk.fill_uniform(torch.empty(plan.n, dtype=torch.float64, device="cuda"), 5)
    f = torch.empty_like(ustar)
    plan.apply(G, M, 1.0, ustar, f, prec=bk.PREC_FP64)
    # the FP64 persistent apply against the oracle (BK5 + mass), first elements of every order
    errs = {}
    Gh_s, Mh_s, uh_s = {}, {}, {}
    for kk, p in enumerate(plan.p):
        q, ns = p + 1, min(plan.E[kk], 64)
        g = G[plan.goff[kk]: plan.goff[kk] + ns * 6 * q ** 3].cpu().numpy().reshape(ns, 6, q, q, q)
        g = g.transpose(0, 3, 4, 1, 2).copy().ravel()   # column (f,k,i,j) -> BK5.cpp's (i,j,f,k)
        m = M[plan.uoff[kk]: plan.uoff[kk] + ns * q ** 3].cpu().numpy()
        uu = ustar[plan.uoff[kk]: plan.uoff[kk] + ns * q ** 3].cpu().numpy()
        ref = oracle.bk5(q, ns, oracle.bk5_matrices(p)[0], g, uu, mass=m, lam=1.0)
        errs[p] = _hostrel(f[plan.uoff[kk]: plan.uoff[kk] + ns * q ** 3].cpu().numpy(), ref)
        Gh_s[p], Mh_s[p], uh_s[p] = g, m, uu
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

    # the per-order launches take KERNEL_AUTO: the kernel shape per order
    # measured by the tuner (sweep or column), FP32 storage and FP64
    shapes = {name: tune.tune_apply(orders, prec=pr, layout=bk.LAYOUT_COLUMN, with_mass=True)
              for name, pr in (("mixed", bk.PREC_MIXED), ("fp64", bk.PREC_FP64))}
    shape_names = {name: {p: ("sweep" if r["kernel"] == bk.KERNEL_SWEEP else "column") for p, r in s.items()}
                   for name, s in shapes.items()}
    aligned = all((o * 8) % 16 == 0 for o in plan.uoff) and all((o * 8) % 16 == 0 for o in plan.goff)
    m_per64 = _events_ms(lambda: per_order(bk.PREC_FP64, G, M, ustar, v64), max(3, steps // 4), 2, torch,
                         graph=True) if aligned else None
    aligned32 = all((o * 4) % 16 == 0 for o in plan.uoff) and all((o * 4) % 16 == 0 for o in plan.goff)
    m_per32 = _events_ms(lambda: per_order(bk.PREC_MIXED, G32, M32, u32, v32), steps, warm, torch, graph=True) \
        if aligned32 else None
    # the column body of the same launch (tiles tuned for it)
    tuned_col = tune.tune(orders, kernel=bk.KERNEL_COLUMN)
    plan_col = tune.make_plan(orders, tuned_col, kernel=bk.KERNEL_COLUMN)
    m_col = _events_ms(lambda: plan_col.apply(G32, M32, 1.0, u32, v32, prec=bk.PREC_MIXED), steps, warm, torch,
                       graph=True)
    plan_col.close()
    # CG to 1e-10: the inner FP32 CG with the Jacobi preconditioner (the
    # solver's default) and without it, each timed after a first solve that
    # builds its graph
    cg_runs = {}
    for name, pc in (("none", hz.PRECOND_NONE), ("jacobi", hz.PRECOND_JACOBI)):
        x = torch.zeros_like(ustar)
        plan.cg(G, M, G32, M32, 1.0, f, x, rtol=1e-10, allow_noconv=True, precond=pc)
        x.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        st = plan.cg(G, M, G32, M32, 1.0, f, x, rtol=1e-10, allow_noconv=True, precond=pc)
        torch.cuda.synchronize()
        cg_runs[name] = dict(st, seconds=time.perf_counter() - t,
                             solution_rel_err=float(torch.linalg.norm(x - ustar) / torch.linalg.norm(ustar)))
    st, solve_s, err = cg_runs["jacobi"], cg_runs["jacobi"]["seconds"], cg_runs["jacobi"]["solution_rel_err"]
    # CPU baseline: the oracle's BK5 + mass on the sampled elements of every order
    units = sum((p + 1) ** 3 * Gh_s[p].size // (6 * (p + 1) ** 3) for p in plan.p)
    sec = _cpu_time(lambda: [oracle.bk5(p + 1, Gh_s[p].size // (6 * (p + 1) ** 3), oracle.bk5_matrices(p)[0],
                                        Gh_s[p], uh_s[p], mass=Mh_s[p], lam=1.0, fast=True) for p in plan.p])
    return {"workload": f"mixed-order Helmholtz p=2..8, E_p=2^(8-p)*{orders[-1][1]} ({plan.n} DoFs), "
                        f"one persistent launch, CG to 1e-10 (FP32 inner, FP64 refinement)",
            "gdofs": plan.n / m_multi / 1e6, "ms_per_apply": m_multi, "dtype": "f32",
            "hbm_frac": 36 * plan.n / m_multi / 1e6 / measured_peak()[0],
            "rel_max_err_vs_oracle_fp64_apply": errs, "oracle_elements_per_order": 64,
            "dofs": plan.n, "tiles": plan.ntiles,
            "tuned": {k: tuned.get(k) for k in ("block", "gstage", "tiles", "evaluated", "starts_ms")},
            "tuned_fp64": {k: tuned64.get(k) for k in ("block", "tiles", "evaluated")},
            "kernel": {bk.KERNEL_SWEEP: "sweep (even-odd)", bk.KERNEL_COLUMN: "column"}[plan.kernel],
            "multi_mixed_gdofs": plan.n / m_multi / 1e6, "multi_fp64_gdofs": plan.n / m_multi64 / 1e6,
            "multi_mixed_column_gdofs": plan.n / m_col / 1e6, "tile_elems_column": tuned_col["tiles"],
            "per_order_mixed_gdofs": (plan.n / m_per32 / 1e6) if m_per32 else None,
            "per_order_fp64_gdofs": (plan.n / m_per64 / 1e6) if m_per64 else None,
            "per_order_kernel_tuned": shape_names,
            # the configuration's comparison: the persistent mixed-precision
            # launch against the plain FP64 per-order launches; and like for
            # like (same precision)
            "speedup_vs_plain_fp64_per_order": ((plan.n / m_multi / 1e6) / (plan.n / m_per64 / 1e6)) if m_per64 else None,
            "ratio_multi_vs_per_order_mixed": (m_per32 / m_multi) if m_per32 else None,
            "ratio_multi_vs_per_order_fp64": (m_per64 / m_multi64) if m_per64 else None,
            "cg": st, "cg_seconds": solve_s, "solution_rel_err": err, "cg_preconditioner": "jacobi",
            "cg_unpreconditioned": cg_runs["none"],
            "cpu_baseline": _cpu_line(units, sec, "BK5 + mass FP64 on the first 64 elements of every order, mean of "
                                                  "3 (oracle/bk_oracle.c, -O3, OpenMP)")}


def headline_parity(D, u, G, v, E, layout, prec, n=1024):
    """max |v - oracle| / max |oracle| over the first and the last n elements
    of the headline apply, the oracle (oracle.bk5, the checker build) run on
    those elements' own u and G."""
    import numpy as np

    import oracle
    Q = P_ORDER + 1
    Q3 = Q ** 3
    n = min(n, E)
    worst, parts = 0.0, {}
    for name, e0 in (("first", 0), ("last", E - n)):
        uh = u[e0 * Q3: (e0 + n) * Q3].double().cpu().numpy()
        g = G[e0 * 6 * Q3: (e0 + n) * 6 * Q3].double().cpu().numpy().reshape(n, 6, Q, Q, Q)
        if layout == 0:      # (f,i,j,k) -> (i,j,f,k)
            g = g.transpose(0, 2, 3, 1, 4)
        elif layout == 2:    # (f,k,i,j) -> (i,j,f,k)
            g = g.transpose(0, 3, 4, 1, 2)
        else:
            g = g.reshape(n, Q, Q, 6, Q)
        ref = oracle.bk5(Q, n, np.asarray(D), np.ascontiguousarray(g).ravel(), uh)
        err = _hostrel(v[e0 * Q3: (e0 + n) * Q3].double().cpu().numpy(), ref)
        parts[name] = err
        worst = max(worst, err)
    return {"rel_max_err_vs_oracle": worst, "elements_checked": {"first": n, "last": n}, "by_range": parts,
            "bound": 1e-12 if prec == 0 else 1e-5,
            "oracle": "oracle/bk_oracle.c: bk::SumFactorization<double, 8> (openmp/BK5.cpp:19-103) restated, "
                      "pinned to the reference's own kernels"}


CONFIG_RUNS = {"bk1": run_bk1, "bk3": run_bk3, "adjoint": run_adjoint, "helmholtz": run_helmholtz}


def run_config_line(args):
    """--workload X: one configuration as its own JSON line."""
    r = CONFIG_RUNS[args.workload](args)
    value = r.get("gdofs", r.get("gpoints_s"))
    ms = r.get("ms_per_apply", r.get("backward_ms"))
    _line(args, r["workload"], value, ms, r.get("dtype", "f64"), {"result": r})


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "bk5":
        run_config_line(args)
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
    # a second sampler over all of this process's GPU work after the input
    # build (the headline, its forms, the end-to-end leg and the other
    # configurations: seconds under load), beside the timed region's own
    clk_all = ClockSampler(local).__enter__()
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
           "config": headline_config(E),
           "options": {"engine": args.engine, "prec": args.prec, "kernel": args.kernel,
                       "layout": f"G6 layout {args.layout} (2: column G(e,f,k,i,j))",
                       "l2": "inputs 8.6 GB >> 129 MB L2, no flush", "parallelism": f"replicas x{world}"},
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
        # both host arrays pinned (empty_like would not pin the second: its
        # copies out would then be synchronous, the host in lockstep with the
        # device, and every host hiccup a gap in the device's work)
        uh = torch.empty(u.numel(), dtype=u.dtype, pin_memory=True)
        vh = torch.empty(u.numel(), dtype=u.dtype, pin_memory=True)
        assert uh.is_pinned() and vh.is_pinned()
        uh.copy_(u)
        hp = bk.HostPlan(5, P_ORDER, E, prec=prec)

        def step_e2e():
            hp.apply(uh, vh, G=G, D=D, engine=engine, layout=args.layout, kernel=kernel, stream=stream)

        # the mean per call (the statistic of `value` and of the reference
        # arm) over at least 200 timed calls after the warm-up (1.4 s), no
        # call left out, every call's own time recorded too: the host link
        # is shared with the machine's other work and stalls one or two calls
        # in most sets of 50 by 20-70 ms, so a short window makes the mean
        # swing between 14 and 19.5 GDoF/s with where the stalls fall
        ncalls = max(steps, 200)
        for _ in range(warmup):
            step_e2e()
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(ncalls + 1)]
        evs[0].record(stream)
        for k in range(ncalls):
            step_e2e()
            evs[k + 1].record(stream)
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        per_call = sorted(evs[k].elapsed_time(evs[k + 1]) for k in range(ncalls))
        te = max_over_ranks(evs[0].elapsed_time(evs[-1]) / 1e3 / ncalls, world)
        e2e_err = float((vh.to(v.device) - v).abs().max())
        hp.close()
        out["e2e"] = {"value": world * dofs / te / 1e9, "unit": UNIT, "h2d_bytes_per_step": u.element_size() * dofs,
                      "d2h_bytes_per_step": u.element_size() * dofs, "ms_per_step": te * 1e3,
                      "calls": ncalls,
                      "per_call_ms": {"min": per_call[0], "median": per_call[len(per_call) // 2],
                                      "max": per_call[-1]},
                      "max_abs_diff_vs_device_apply": e2e_err,
                      "note": "bk5_apply_host: G (6.4 GB) resident on the device; u in, v out every step "
                              "from/to pinned host memory in 16 element chunks, copies overlapping the applies"}

    # the forms side by side, with their error against the FP64 result
    if not args.no_forms and rank == 0 and prec == bk.PREC_FP64:
        forms = {}
        ref = v.clone()
        forms["fp64_ff"] = {"gdofs": value / world}
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
        for name, pr in (("mixed_fp32_storage", bk.PREC_MIXED), ("fp32", bk.PREC_FP32)):
            tm = time_loop(lambda: bk.bk5_apply(P_ORDER, E, D, G32, u32, v32, prec=pr, layout=args.layout,
                                                stream=stream),
                           max(3, steps // 4), 3, 1, stream, torch)
            err = float((v32.double() - ref).abs().max() / ref.abs().max())
            # against the FP64 oracle on the FP64 inputs (storage rounding included)
            orc = headline_parity(D, u, G, v32, E, args.layout, bk.PREC_FP64)["rel_max_err_vs_oracle"]
            forms[name] = {"gdofs": dofs / tm / 1e9, "rel_err_vs_fp64": err, "rel_err_vs_oracle": orc,
                           "speedup_vs_fp64": (dofs / tm / 1e9) / (value / world),
                           "hbm_frac": 4 * 8 * dofs / tm / 1e9 / peak}
        out["forms"] = forms
        del u32, G32, v32

    # the headline's own result against the FP64 oracle: the first and the
    # last elements of u and G copied to the host (G relaid to BK5.cpp's
    # interleaved layout), oracle.bk5 on them
    if rank == 0:
        out["parity"] = headline_parity(D, u, G, v, E, args.layout, prec)
        if "forms" in out:
            out["forms"]["fp64_ff"]["rel_err_vs_oracle"] = out["parity"]["rel_max_err_vs_oracle"]

    if rank == 0 and world == 1 and not args.no_configs and E == E_FULL:
        out["configs"] = {}
        for name, fn in CONFIG_RUNS.items():
            try:
                out["configs"][name] = fn(args)
            except Exception as exc:   # recorded, so that the headline line still prints
                out["configs"][name] = {"error": f"{type(exc).__name__}: {exc}"}
            torch.cuda.synchronize()
            torch.cuda.empty_cache()

    clk_all.__exit__(None, None, None)
    out["clocks_gpu_work"] = dict(clk_all.summary(), note="every GPU phase of this run after the input build")
    if rank == 0 and world == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_bk5_run(E, 3, 1)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
