"""Times one 1-D contraction (Q = 8, the BK5 p = 7 GLL derivative) in FP64
accuracy by the probe's routes (include/bk_probe.h) on the same lines:

    python -m omp_bk_gb300.contract_probe [--lines N] [--reps R]

The lines (64 B in, 64 B out each) are sized to stay in the 129 MB L2 by
default, so that the routes' arithmetic, not HBM, sets the time.  Prints one
JSON line: per route the time per launch (CUDA events, mean of R launches
after 3 warm-up launches), outputs per second and the largest error against
numpy's FP64 product, normwise per line (|y - ref| / (sum_n |D(i,n)|
max_n |x(n)|)); and the
difference of each route's time from the copy route's (the contraction
itself)."""
from __future__ import annotations

import argparse
import json

import numpy as np


def main(argv=None):
    import torch

    import omp_bk_gb300 as bk
    ap = argparse.ArgumentParser()
    ap.add_argument("--lines", type=int, default=1 << 19)
    ap.add_argument("--reps", type=int, default=50)
    a = ap.parse_args(argv)
    n = (a.lines // 16) * 16
    D = bk.bk5_matrices(7)[0]
    x = torch.empty(n * 8, dtype=torch.float64, device="cuda")
    bk.fill_uniform(x, 77)
    y = torch.empty_like(x)
    xs = x[: 4096 * 8].cpu().numpy().reshape(-1, 8)
    Dm = D.reshape(8, 8)
    ref = xs @ Dm.T
    bound = np.abs(Dm).sum(axis=1)[None, :] * np.abs(xs).max(axis=1)[:, None]
    out = {"lines": n, "outputs_per_launch": n * 8, "reps": a.reps}
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for name, m in (("copy", bk.PROBE_COPY), ("ff", bk.PROBE_FF), ("mma", bk.PROBE_MMA)):
        for _ in range(3):
            bk.probe_contract(m, D, x, y)
        torch.cuda.synchronize()
        t0.record()
        for _ in range(a.reps):
            bk.probe_contract(m, D, x, y)
        t1.record()
        torch.cuda.synchronize()
        ms = t0.elapsed_time(t1) / a.reps
        got = y[: 4096 * 8].cpu().numpy().reshape(-1, 8)
        err = float(np.max(np.abs(got - (xs if name == "copy" else ref)) / (np.abs(xs) if name == "copy" else bound)))
        out[name] = {"us_per_launch": ms * 1e3, "goutputs_s": n * 8 / ms / 1e6, "max_normwise_err": err}
    for name in ("ff", "mma"):
        out[name]["contraction_us"] = out[name]["us_per_launch"] - out["copy"]["us_per_launch"]
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
