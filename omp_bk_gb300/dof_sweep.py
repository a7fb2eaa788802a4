"""Throughput versus problem size: the DoF sweep of the reference's study
scripts (scripts/study/dof_sweep.sh) for the CUDA operators.

For each operator (BK1, BK3, BK5), order p and arithmetic form, the element
count runs log-spaced over [dof_min, dof_max] DoFs (ppd points per decade;
the reference's formula: round(10^(lo + i/ppd) / nodes^3), duplicates
dropped), and each point is timed as the reference times a kernel -- the
best of `ntests` single applies, host wall time around the call and a
stream synchronize (bk_common.h time_min) -- and with CUDA events on the
device.  The CSV has the reference's columns

    api,nq,kernel,nelmt,dofs,gdofs,gbs,gdofs_dev,gbs_dev

(api = cuda; nq = quadrature points per direction; GB/s in the reference's
convention sizeof(T) (2 in + JxW|G), BK1.cpp:32, BK5.cpp:144), and
<out>.stream holds the STREAM copy and triad bandwidths of the same run.
The sweep shows the launch-latency floor at small E and the L2 -> HBM
transition (129 MB L2).

    python -m omp_bk_gb300.dof_sweep --bk 5 --p 3,5,7 --out bk5_sweep.csv
"""
from __future__ import annotations

import argparse
import math
import sys
import time

FORMS = {
    # name: (prec, engine, bytes per value)
    "ff": ("PREC_FP64", "ENGINE_FF", 8),
    "dfma": ("PREC_FP64", "ENGINE_DFMA", 8),
    "mixed": ("PREC_MIXED", "ENGINE_AUTO", 4),
    "fp32": ("PREC_FP32", "ENGINE_AUTO", 4),
}

HEADER = "api,nq,kernel,nelmt,dofs,gdofs,gbs,gdofs_dev,gbs_dev"


def nodes_per_dim(bk: int, p: int) -> int:
    """DoF nodes per direction: GLL nodes P = p + 1 (BK1, BK3), GLL points
    Q = p + 1 (BK5)."""
    return p + 1


def quad_per_dim(bk: int, p: int) -> int:
    """Quadrature points per direction: Q = p + 2 Gauss (BK1, BK3), p + 1
    GLL (BK5)."""
    return p + 2 if bk in (1, 3) else p + 1


def element_counts(nodes: int, dof_min: float, dof_max: float, ppd: int):
    """Distinct element counts for the log-spaced DoF targets, ascending."""
    lo, hi, n3 = math.log10(dof_min), math.log10(dof_max), nodes ** 3
    n = round((hi - lo) * ppd)
    return sorted({max(1, round(10 ** (lo + i / ppd) / n3)) for i in range(n + 1)})


def values_per_element(bk: int, p: int):
    """(u/v values, geometric values) per element."""
    P, Q = nodes_per_dim(bk, p), quad_per_dim(bk, p)
    if bk == 1:
        return P ** 3, Q ** 3
    return P ** 3, 6 * Q ** 3


def _sweep_point(bk_mod, torch, bk, p, form, E, ntests, stream, kernel="auto", layout=1):
    prec_name, eng_name, vb = FORMS[form]
    prec, engine = getattr(bk_mod, prec_name), getattr(bk_mod, eng_name)
    dt = torch.float64 if vb == 8 else torch.float32
    nuv, ngeo = values_per_element(bk, p)
    u = bk_mod.fill_uniform(torch.empty(E * nuv, dtype=dt, device="cuda"), 1)
    g = bk_mod.fill_uniform(torch.empty(E * ngeo, dtype=dt, device="cuda"), 2, 0.5, 1.5)
    v = torch.empty_like(u)
    if bk == 1:
        B = bk_mod.bk1_bk3_matrices(p)[0]
        call = lambda: bk_mod.bk1_apply(p, E, B, g, u, v, prec=prec, engine=engine, stream=stream)
    elif bk == 3:
        B, D = bk_mod.bk1_bk3_matrices(p)[:2]
        call = lambda: bk_mod.bk3_apply(p, E, B, D, g, u, v, prec=prec, engine=engine, stream=stream)
    else:
        D = bk_mod.bk5_matrices(p)[0]
        kern = {"auto": bk_mod.KERNEL_AUTO, "sweep": bk_mod.KERNEL_SWEEP, "column": bk_mod.KERNEL_COLUMN}[kernel]
        call = lambda: bk_mod.bk5_apply(p, E, D, g, u, v, prec=prec, engine=engine, kernel=kern, layout=layout,
                                        stream=stream)
    call()
    torch.cuda.synchronize()
    best_host = best_dev = float("inf")
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    for _ in range(ntests):
        t = time.perf_counter()
        ev0.record(stream)
        call()
        ev1.record(stream)
        stream.synchronize()
        best_host = min(best_host, time.perf_counter() - t)
        best_dev = min(best_dev, ev0.elapsed_time(ev1) * 1e-3)
    bytes_ = vb * E * (2 * nuv + ngeo)
    dofs = E * nuv
    return dofs, dofs / best_host / 1e9, bytes_ / best_host / 1e9, dofs / best_dev / 1e9, bytes_ / best_dev / 1e9


def stream_lines(bk_mod, torch, nbytes=1 << 30):
    """STREAM copy and triad bandwidth (GB/s, best of 10) over nbytes per array."""
    n = nbytes // 8
    a, b, c = (torch.ones(n, dtype=torch.float64, device="cuda") for _ in range(3))
    out = []
    for name, kind, arrays in (("copy", 0, 2), ("triad", 1, 3)):
        best = float("inf")
        for _ in range(10):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            bk_mod.stream_kernel(kind, a, b, c)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) * 1e-3)
        out.append(f"{name} {arrays * nbytes / best / 1e9:.1f} GB/s")
    return out


def parse(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--bk", default="5", help="operators, comma separated (1, 3, 5)")
    ap.add_argument("--p", default="2,4,6", help="orders, comma separated")
    ap.add_argument("--kernels", default="ff,mixed", help="forms: ff, dfma, mixed, fp32")
    ap.add_argument("--kernel", default="auto", choices=("auto", "sweep", "column"),
                    help="BK5 kernel shape (bk_kernel_shape)")
    ap.add_argument("--layout", type=int, default=1, choices=(0, 1, 2),
                    help="BK5 G layout (bk_layout; 1 = BK5.cpp's interleaved layout)")
    ap.add_argument("--dof-min", type=float, default=1e3)
    ap.add_argument("--dof-max", type=float, default=1e8)
    ap.add_argument("--ppd", type=int, default=4, help="points per decade")
    ap.add_argument("--ntests", type=int, default=20)
    ap.add_argument("--out", default="dof_sweep.csv")
    return ap.parse_args(argv)


def main(argv=None):
    args = parse(argv)
    import torch

    import omp_bk_gb300 as bk_mod
    if not torch.cuda.is_available():
        raise SystemExit("dof_sweep needs a CUDA device")
    stream = torch.cuda.current_stream()
    rows = [HEADER]
    print(HEADER)
    for bk in (int(x) for x in args.bk.split(",")):
        for p in (int(x) for x in args.p.split(",")):
            nq = quad_per_dim(bk, p)
            for form in args.kernels.split(","):
                if form not in FORMS:
                    raise SystemExit(f"unknown form {form!r}")
                for E in element_counts(nodes_per_dim(bk, p), args.dof_min, args.dof_max, args.ppd):
                    dofs, g, gb, gd, gbd = _sweep_point(bk_mod, torch, bk, p, form, E, args.ntests, stream,
                                                        args.kernel, args.layout)
                    row = f"cuda,{nq},bk{bk}_{form},{E},{dofs},{g:.4f},{gb:.2f},{gd:.4f},{gbd:.2f}"
                    rows.append(row)
                    print(row, flush=True)
    with open(args.out, "w") as f:
        f.write("\n".join(rows) + "\n")
    with open(args.out + ".stream", "w") as f:
        f.write("\n".join(stream_lines(bk_mod, torch)) + "\n")
    return 0


if __name__ == "__main__":
    sys.exit(main())
