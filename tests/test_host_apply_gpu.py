"""The applies on host arrays (include/bk_host.h): element chunks copied in,
applied and copied out on three streams must give exactly the device
apply's result, for every operator, ragged chunk counts, pinned and pageable
host memory, and consecutive calls that reuse the device slots."""
import numpy as np
import pytest
import torch

from gpu_util import dev, host, random_case

pytestmark = pytest.mark.gpu


def _dt(bk, prec):
    return torch.float64 if prec == bk.PREC_FP64 else torch.float32


@pytest.mark.parametrize("op,p,E,chunk", [(5, 7, 37, 0), (5, 2, 23, 3), (5, 8, 9, 2), (3, 6, 19, 4), (3, 1, 30, 0),
                                          (1, 3, 41, 5), (1, 8, 7, 0)])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_host_apply_matches_device_apply(bklib, op, p, E, chunk, prec):
    bk = bklib
    pr = bk.PREC_FP64 if prec == "fp64" else bk.PREC_MIXED
    dt = _dt(bk, pr)
    nq, basis, dbasis, g, u = random_case(op, p, E)
    gd = dev(g, "f64" if dt == torch.float64 else "f32")
    ud = dev(u, "f64" if dt == torch.float64 else "f32")
    ref = torch.empty_like(ud)
    k = None
    if op == 1:
        bk.bk1_apply(p, E, basis, gd, ud, ref, prec=pr)
    elif op == 3:
        k = torch.exp(torch.linspace(-1, 1, E * nq ** 3, dtype=dt, device="cuda"))
        bk.bk3_apply(p, E, basis, dbasis, gd, ud, ref, k=k, prec=pr)
    else:
        bk.bk5_apply(p, E, dbasis, gd, ud, ref, prec=pr)
    plan = bk.HostPlan(op, p, E, prec=pr, chunk_elems=chunk)
    try:
        uh = ud.cpu().pin_memory()
        vh = torch.full_like(uh, float("nan")).pin_memory()
        plan.apply(uh, vh, G=gd, B=basis, D=dbasis, k=k)
        torch.cuda.synchronize()
        assert torch.equal(vh, ref.cpu())
        # pageable numpy arrays, twice in a row with different inputs
        un = host(ud).astype(np.float64 if dt == torch.float64 else np.float32)
        vn = np.full_like(un, np.nan)
        plan.apply(2 * un, vn, G=gd, B=basis, D=dbasis, k=k)
        plan.apply(un, vn, G=gd, B=basis, D=dbasis, k=k)
        torch.cuda.synchronize()
        assert np.array_equal(vn, host(ref).astype(vn.dtype))
    finally:
        plan.close()


def test_host_apply_argument_checks(bklib):
    bk = bklib
    D = bk.bk5_matrices(3)[0]
    plan = bk.HostPlan(5, 3, 0)
    try:
        plan.apply(np.zeros(0), np.zeros(0), G=None, D=D)   # E = 0: nothing to do
    finally:
        plan.close()
    G = torch.zeros(4 * 6 * 64, dtype=torch.float64, device="cuda")
    u, v = np.zeros(4 * 64), np.zeros(4 * 64)
    p3 = bk.HostPlan(3, 3, 4)
    try:
        with pytest.raises(bk.BKError, match="bk5_apply_host"):
            p3.op = 5                  # a BK3 plan used for BK5: rejected by the library
            p3.apply(u, v, G=G, D=D)
    finally:
        p3.op = 3
        p3.close()
    p5 = bk.HostPlan(5, 3, 4, prec=bk.PREC_FP64)
    try:
        p5.prec = bk.PREC_MIXED        # options precision other than the plan's
        with pytest.raises(bk.BKError):
            p5.apply(u, v, G=G, D=D)
    finally:
        p5.close()
    with pytest.raises(bk.BKError):
        bk.HostPlan(4, 3, 4)          # no operator 4
    with pytest.raises(bk.BKError):
        bk.HostPlan(5, 9, 4)          # order outside 1..8
