"""Shared helpers of the GPU tests: device tensors and the reference's test
data."""
import numpy as np

import oracle


def dev(a, dtype):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(np.asarray(a), dtype=np.float64 if dtype == "f64" else np.float32))
    return t.cuda()


def host(t):
    return t.detach().cpu().numpy().astype(np.float64)


def sizes(bk, p):
    nq = p + 1 if bk == 5 else p + 2
    nm = nq if bk == 5 else nq - 1
    ngeo = nq ** 3 if bk == 1 else 6 * nq ** 3
    return nq, nm, ngeo


def random_case(bk, p, E, seed=12345):
    """The reference's random test data (LCG, include/bk_common.h:92-107) and
    cos test basis: (nq, basis, dbasis, geo, u) in double."""
    nq, nm, ngeo = sizes(bk, p)
    u, g = oracle.random_test_data(E * nm ** 3, E * ngeo, seed)
    basis = oracle.test_basis(nm, nq) if bk != 5 else None
    dbasis = oracle.test_basis(nq, nq) if bk != 1 else None
    return nq, basis, dbasis, g, u


def oracle_apply(bk, nq, E, basis, dbasis, g, u, k=None, mass=None, lam=0.0):
    if bk == 1:
        return oracle.bk1(nq, E, basis, g, u)
    if bk == 3:
        return oracle.bk3(nq, E, basis, dbasis, g, u, k=k)
    return oracle.bk5(nq, E, dbasis, g, u, mass=mass, lam=lam)


def gpu_apply(bklib, bk, p, E, basis, dbasis, g, u, prec, engine=0, layout=1, nfactors=6, k=None, mass=None,
              lam=0.0):
    """Runs the CUDA path through the C ABI; returns the output on the host."""
    import torch
    dt = "f64" if prec == bklib.PREC_FP64 else "f32"
    gu, gg = dev(u, dt), dev(g, dt)
    out = torch.full_like(gu, float("nan"))   # poisoned: a missed output shows
    if bk == 1:
        bklib.bk1_apply(p, E, basis, gg, gu, out, prec=prec, engine=engine)
    elif bk == 3:
        bklib.bk3_apply(p, E, basis, dbasis, gg, gu, out, k=None if k is None else dev(k, dt), prec=prec,
                        engine=engine)
    else:
        bklib.bk5_apply(p, E, dbasis, gg, gu, out, prec=prec, engine=engine, layout=layout, nfactors=nfactors,
                        mass=None if mass is None else dev(mass, dt), lam=lam)
    torch.cuda.synchronize()
    return host(out)
