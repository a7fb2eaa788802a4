"""The batched mixed-order Helmholtz operator (one persistent launch over
orders p = 2..8) and its mixed-precision CG with FP64 refinement.

  - the persistent apply equals the per-order BK5 apply with the mass term
    (FP64: < 1e-12 relative; FP32 storage: < 1e-5) and the oracle's FP64
    BK5 + lambda mass (oracle/bk_oracle.c);
  - CG reaches |f - A x| <= 1e-10 |f| (FP64 residual), checked again with the
    oracle's FP64 operator on the host.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import oracle
from gpu_util import host

pytestmark = pytest.mark.gpu


def _slices(plan, k):
    q = plan.p[k] + 1
    E = plan.E[k]
    return (slice(plan.uoff[k], plan.uoff[k] + E * q ** 3), slice(plan.goff[k], plan.goff[k] + 6 * E * q ** 3))


def _col_to_interleaved(Gc, E, q):
    """G(e, f, k, i, j) -> G(e, i, j, f, k)."""
    return np.ascontiguousarray(Gc.reshape(E, 6, q, q, q).transpose(0, 3, 4, 1, 2)).ravel()


@pytest.fixture(scope="module")
def small_plan(bklib):
    from omp_bk_gb300.helmholtz import HelmholtzPlan
    orders = [(p, 5 + 2 * p) for p in range(2, 9)]
    plan = HelmholtzPlan(orders)
    G, M = plan.geometry(seed=3)
    u = bklib.fill_uniform(torch.empty(plan.n, dtype=torch.float64, device="cuda"), 4)
    yield plan, G, M, u
    plan.close()


@pytest.mark.parametrize("kernel", ["sweep", "column"])
@pytest.mark.parametrize("prec", ["ff", "dfma", "mixed", "fp32"])
def test_multi_apply_matches_per_order(bklib, small_plan, prec, kernel):
    bk = bklib
    plan, G, M, u = small_plan
    assert plan.kernel == bk.KERNEL_SWEEP   # GLL derivatives: even-odd body by default
    plan.set_kernel(bk.KERNEL_SWEEP if kernel == "sweep" else bk.KERNEL_COLUMN)
    assert plan.kernel == (bk.KERNEL_SWEEP if kernel == "sweep" else bk.KERNEL_COLUMN)
    lam = 1.0 if prec != "dfma" else 0.75
    if prec in ("ff", "dfma"):
        pr, eng, dt, tol = bk.PREC_FP64, (bk.ENGINE_FF if prec == "ff" else bk.ENGINE_DFMA), torch.float64, 1e-12
    else:
        pr, eng, dt, tol = (bk.PREC_MIXED if prec == "mixed" else bk.PREC_FP32), 0, torch.float32, 1e-5
    Gd, Md, ud = G.to(dt), M.to(dt), u.to(dt)
    v = torch.full_like(ud, float("nan"))
    plan.apply(Gd, Md, lam, ud, v, prec=pr, engine=eng)
    torch.cuda.synchronize()
    for k, p in enumerate(plan.p):
        su, sg = _slices(plan, k)
        D, _, _ = bk.bk5_matrices(p)
        w = torch.full_like(ud[su], float("nan"))
        # the per-order entry point wants 16-byte aligned arrays: copies
        bk.bk5_apply(p, plan.E[k], D, Gd[sg].clone(), ud[su].clone(), w, prec=pr, engine=eng,
                     layout=bk.LAYOUT_COLUMN, mass=Md[su].clone(), lam=lam)
        torch.cuda.synchronize()
        assert oracle.rel_maxdiff(host(v[su]), host(w)) < tol, p
        # the oracle: FP64 BK5 on the same (rounded) inputs, G interleaved
        q = p + 1
        f = (lambda a: host(a)) if dt == torch.float64 else (lambda a: host(a).astype(np.float32).astype(np.float64))
        ref = oracle.bk5(q, plan.E[k], D, _col_to_interleaved(f(Gd[sg]), plan.E[k], q), f(ud[su]),
                         mass=f(Md[su]), lam=lam)
        assert oracle.rel_maxdiff(host(v[su]), ref) < tol, p
    plan.set_kernel(bk.KERNEL_AUTO)


def test_sweep_needs_centro_antisymmetric_D(bklib):
    """A D that is not centro-antisymmetric keeps the column body."""
    import ctypes as C
    from omp_bk_gb300.helmholtz import HelmholtzPlan, OrderRange, _declare
    plan = HelmholtzPlan([(3, 4)])
    assert plan.kernel == bklib.KERNEL_SWEEP
    plan.close()
    L = _declare()
    D = np.arange(16, dtype=np.float64) / 7.0
    rng = (OrderRange * 1)(OrderRange(3, 4, 0))
    dp = (C.POINTER(C.c_double) * 1)(D.ctypes.data_as(C.POINTER(C.c_double)))
    h = C.c_void_p()
    assert L.bk_hplan_create(C.byref(h), 1, rng, dp, None) == bklib.BK_OK
    try:
        assert L.bk_hplan_size(h, 3) == bklib.KERNEL_COLUMN
        assert L.bk_hplan_set_kernel(h, bklib.KERNEL_SWEEP) == bklib.BK_ERR_ARG
        assert L.bk_hplan_set_kernel(h, bklib.KERNEL_AUTO) == bklib.BK_OK
        assert L.bk_hplan_size(h, 3) == bklib.KERNEL_COLUMN
    finally:
        L.bk_hplan_destroy(h)


def test_cg_converges(bklib, small_plan):
    bk = bklib
    plan, G, M, ustar = small_plan
    f = torch.empty_like(ustar)
    plan.apply(G, M, 1.0, ustar, f, prec=bk.PREC_FP64)
    x = torch.zeros_like(ustar)
    st = plan.cg(G, M, G.float(), M.float(), 1.0, f, x, rtol=1e-10)
    torch.cuda.synchronize()
    assert st["converged"] and st["relres"] <= 1e-10, st
    assert st["outer"] >= 1 and st["inner"] >= 1
    # FP64 residual on the host with the oracle
    r2 = 0.0
    for k, p in enumerate(plan.p):
        su, sg = _slices(plan, k)
        q = p + 1
        D, _, _ = bk.bk5_matrices(p)
        Ax = oracle.bk5(q, plan.E[k], D, _col_to_interleaved(host(G[sg]), plan.E[k], q), host(x[su]),
                        mass=host(M[su]), lam=1.0)
        r2 += float(np.sum((host(f[su]) - Ax) ** 2))
    assert np.sqrt(r2) <= 2e-10 * float(torch.linalg.norm(f))
    assert float(torch.linalg.norm(x - ustar) / torch.linalg.norm(ustar)) < 1e-6


def test_cg_graph_reused_and_restarted(bklib, small_plan):
    """A second solve reuses the captured graph; a warm start converges in
    fewer refinement steps."""
    bk = bklib
    plan, G, M, ustar = small_plan
    f = torch.empty_like(ustar)
    plan.apply(G, M, 1.0, ustar, f, prec=bk.PREC_FP64)
    G32, M32 = G.float(), M.float()
    x = torch.zeros_like(ustar)
    a = plan.cg(G, M, G32, M32, 1.0, f, x, rtol=1e-10)
    b = plan.cg(G, M, G32, M32, 1.0, f, x, rtol=1e-10)
    assert a["converged"] and b["converged"]
    assert b["outer"] == 0 and b["relres"] <= 1e-10


def test_tuner(bklib):
    """The tuner's plan shape: a block size and a G staging from its lists,
    per-order tiles from their candidates (lines within the plan limit); the
    plan it describes applies the operator."""
    from omp_bk_gb300 import tune
    orders = [(2, 512), (5, 256), (8, 64)]
    best = tune.tune(orders, max_elements=512, reps=2, use_cache=False)
    assert best["block"] in tune.BLOCKS and best["gstage"] in tune.GSTAGE and best["ms"] > 0
    assert best["evaluated"] >= len(tune.BLOCKS) * len(tune.GSTAGE)
    for p in (2, 5, 8):
        eb = best["tiles"][p]
        assert eb in tune.candidates(p, best["block"]) and eb * (p + 1) ** 2 <= tune.MAX_TILE_LINES
    col = tune.tune(orders, max_elements=512, reps=2, use_cache=False, kernel=bklib.KERNEL_COLUMN)
    assert col["block"] == 0
    for p in (2, 5, 8):
        assert col["tiles"][p] in tune.candidates(p) and col["tiles"][p] * (p + 1) ** 2 <= 256
    # the FP64-storage launches tuned apart, and given to the plan
    b64 = tune.tune(orders, prec=bklib.PREC_FP64, max_elements=512, reps=2, use_cache=False)
    assert b64["block"] in tune.BLOCKS and b64["gstage"] == 0
    for p in (2, 5, 8):
        assert b64["tiles"][p] in tune.candidates(p, b64["block"])
    plan = tune.make_plan(orders, best, fp64=b64)
    try:
        assert plan.block == best["block"] and plan.gstage == best["gstage"]
        assert plan.fp64_block == b64["block"]
        assert plan.fp64_ntiles == sum(-(-E // b64["tiles"][p]) for p, E in orders)
        G, M = plan.geometry(seed=8)
        u = bklib.fill_uniform(torch.empty(plan.n, dtype=torch.float64, device="cuda"), 9)
        _check_per_order(bklib, plan, G, M, u, "ff")
        _check_per_order(bklib, plan, G, M, u, "mixed")
    finally:
        plan.close()


def _check_per_order(bk, plan, G, M, u, prec, lam=1.0):
    """The plan's persistent apply against the per-order BK5 applies with
    the mass term and, on each order's first elements, the oracle."""
    if prec in ("ff", "dfma"):
        pr, eng, dt, tol = bk.PREC_FP64, (bk.ENGINE_FF if prec == "ff" else bk.ENGINE_DFMA), torch.float64, 1e-12
    else:
        pr, eng, dt, tol = (bk.PREC_MIXED if prec == "mixed" else bk.PREC_FP32), 0, torch.float32, 1e-5
    Gd, Md, ud = G.to(dt), M.to(dt), u.to(dt)
    v = torch.full_like(ud, float("nan"))
    plan.apply(Gd, Md, lam, ud, v, prec=pr, engine=eng)
    torch.cuda.synchronize()
    for k, p in enumerate(plan.p):
        su, sg = _slices(plan, k)
        D, _, _ = bk.bk5_matrices(p)
        w = torch.full_like(ud[su], float("nan"))
        bk.bk5_apply(p, plan.E[k], D, Gd[sg].clone(), ud[su].clone(), w, prec=pr, engine=eng,
                     layout=bk.LAYOUT_COLUMN, mass=Md[su].clone(), lam=lam)
        torch.cuda.synchronize()
        assert oracle.rel_maxdiff(host(v[su]), host(w)) < tol, p
        q, E = p + 1, min(plan.E[k], 64)
        f = (lambda a: host(a)) if dt == torch.float64 else (lambda a: host(a).astype(np.float32).astype(np.float64))
        ref = oracle.bk5(q, E, D, _col_to_interleaved(f(Gd[sg][: 6 * E * q ** 3]), E, q), f(ud[su][: E * q ** 3]),
                         mass=f(Md[su][: E * q ** 3]), lam=lam)
        assert oracle.rel_maxdiff(host(v[su][: E * q ** 3]), ref) < tol, p


@pytest.mark.parametrize("prec", ["ff", "dfma", "mixed", "fp32"])
@pytest.mark.parametrize("shape", ["many_tiles", "many_tiles_gstage", "looped_lines", "looped_lines_gstage"])
def test_multi_apply_tile_shapes(bklib, prec, shape):
    """Blocks that walk several tiles each (FP32 storage: the next tile's u
    and mass staged into the second buffer while the current tile computes,
    its G prefetched into L2 or staged after the pointwise stage; FP64: the
    single stage refilled), and tiles with more lines than the block has
    threads (bk_hplan_set_shape): the persistent apply equals the per-order
    applies and the oracle."""
    from omp_bk_gb300.helmholtz import HelmholtzPlan
    gstage = int(shape.endswith("gstage"))
    if shape.startswith("many_tiles"):
        plan = HelmholtzPlan([(p, 700, 1) for p in range(2, 9)], gstage=gstage)
        assert plan.ntiles > 3 * 1216   # more tiles than resident blocks
    else:
        # 180, 180 and 243 lines per tile, swept by 64 threads
        plan = HelmholtzPlan([(2, 300, 20), (5, 90, 5), (8, 40, 3)], block=64, gstage=gstage)
        assert plan.smem_bytes(fp64=True) <= 232448 and plan.block == 64
    assert plan.gstage == gstage
    try:
        G, M = plan.geometry(seed=12)
        u = bklib.fill_uniform(torch.empty(plan.n, dtype=torch.float64, device="cuda"), 13)
        _check_per_order(bklib, plan, G, M, u, prec, lam=1.0 if prec != "dfma" else 0.5)
    finally:
        plan.close()


def test_cg_with_shapes(bklib):
    """The CG (its inner graph fuses p . Ap into the FP32 apply) on a plan
    with a block smaller than its tiles and G staged."""
    from omp_bk_gb300.helmholtz import HelmholtzPlan
    plan = HelmholtzPlan([(2, 60, 20), (4, 30, 6), (7, 12, 2)], block=64, gstage=1)
    try:
        G, M = plan.geometry(seed=14)
        ustar = bklib.fill_uniform(torch.empty(plan.n, dtype=torch.float64, device="cuda"), 15)
        f = torch.empty_like(ustar)
        plan.apply(G, M, 1.0, ustar, f, prec=bklib.PREC_FP64)
        x = torch.zeros_like(ustar)
        st = plan.cg(G, M, G.float(), M.float(), 1.0, f, x, rtol=1e-10)
        torch.cuda.synchronize()
        assert st["converged"] and st["relres"] <= 1e-10, st
        assert float(torch.linalg.norm(x - ustar) / torch.linalg.norm(ustar)) < 1e-6
    finally:
        plan.close()


def test_set_shape_arguments(bklib):
    from omp_bk_gb300.helmholtz import HelmholtzPlan, _declare
    L = _declare()
    plan = HelmholtzPlan([(3, 10, 40)])   # 640 lines per tile: not for the column body
    try:
        for bad in ((32, 0), (48, 0), (100, 0), (288, 0), (64, 2), (0, -1)):
            assert L.bk_hplan_set_shape(plan.h, *bad) == bklib.BK_ERR_ARG
        for good in ((0, 0), (64, 1), (96, 0), (256, 1)):
            assert L.bk_hplan_set_shape(plan.h, *good) == bklib.BK_OK
        assert plan.block == 256 and plan.gstage == 1
        assert L.bk_hplan_set_kernel(plan.h, bklib.KERNEL_COLUMN) == bklib.BK_ERR_ARG
    finally:
        plan.close()


def test_fp64_shape(bklib):
    """The FP64-storage launches on their own tiles and threads
    (bk_hplan_set_fp64_shape): the same results bit for bit (an element's
    arithmetic does not depend on its tile), the FP32 launches untouched,
    the CG (FP64 residual on the FP64 tiles) still converging, and the
    arguments checked."""
    from omp_bk_gb300.helmholtz import HelmholtzPlan, _declare
    L = _declare()
    plan = HelmholtzPlan([(2, 200, 20), (5, 40, 3), (8, 9, 1)], block=128)
    try:
        G, M = plan.geometry(seed=16)
        u = bklib.fill_uniform(torch.empty(plan.n, dtype=torch.float64, device="cuda"), 17)
        G32, M32, u32 = G.float(), M.float(), u.float()
        outs = {}
        for name in ("plain", "own", "back"):
            if name == "own":
                plan.set_fp64_shape({2: 7, 5: 0, 8: 2}, 96)
                assert plan.fp64_block == 96 and plan.block == 128
                assert plan.fp64_ntiles == 29 + 14 + 5 and plan.ntiles == 10 + 14 + 9
            elif name == "back":
                plan.set_fp64_shape(None)
                assert plan.fp64_block == 128 and plan.fp64_ntiles == plan.ntiles
            r = {}
            for key, prec, eng, GG, MM, uu in (("ff", bklib.PREC_FP64, bklib.ENGINE_FF, G, M, u),
                                              ("dfma", bklib.PREC_FP64, bklib.ENGINE_DFMA, G, M, u),
                                              ("mixed", bklib.PREC_MIXED, bklib.ENGINE_AUTO, G32, M32, u32)):
                v = torch.full_like(uu, float("nan"))
                plan.apply(GG, MM, 1.0, uu, v, prec=prec, engine=eng)
                torch.cuda.synchronize()
                r[key] = v
            outs[name] = r
        for key in ("ff", "dfma", "mixed"):
            assert torch.equal(outs["plain"][key], outs["own"][key]), key
            assert torch.equal(outs["plain"][key], outs["back"][key]), key
        plan.set_fp64_shape({2: 7, 5: 2, 8: 2}, 64)
        f = torch.empty_like(u)
        plan.apply(G, M, 1.0, u, f, prec=bklib.PREC_FP64)
        x = torch.zeros_like(u)
        st = plan.cg(G, M, G32, M32, 1.0, f, x, rtol=1e-10)
        torch.cuda.synchronize()
        assert st["converged"] and st["relres"] <= 1e-10, st
        for bad_tiles, bad_block in (([0, 0, 13], 0), ([-1, 0, 0], 0), ([0, 0, 0], 32), ([0, 0, 0], 100)):
            arr = (C.c_int * 3)(*bad_tiles)
            assert L.bk_hplan_set_fp64_shape(plan.h, arr, bad_block, None) == bklib.BK_ERR_ARG
        assert plan.fp64_block == 64   # a refused shape changes nothing
    finally:
        plan.close()


def test_operator_spd(bklib, small_plan):
    """K + lambda M is symmetric positive definite: u.Au >= lambda u.Mu > 0
    (K positive semi-definite, the GLL mass positive) and u.Aw = w.Au."""
    bk = bklib
    plan, G, M, _ = small_plan
    lam = 1.0
    for seed in (21, 22, 23):
        u = bk.fill_uniform(torch.empty(plan.n, dtype=torch.float64, device="cuda"), seed)
        w = bk.fill_uniform(torch.empty_like(u), seed + 100)
        Au, Aw = torch.empty_like(u), torch.empty_like(u)
        plan.apply(G, M, lam, u, Au, prec=bk.PREC_FP64)
        plan.apply(G, M, lam, w, Aw, prec=bk.PREC_FP64)
        torch.cuda.synchronize()
        uAu = float(torch.dot(u, Au))
        uMu = float(torch.dot(u, M * u))
        assert uMu > 0 and uAu >= lam * uMu * (1 - 1e-12)
        scale = float(torch.linalg.norm(u) * torch.linalg.norm(Aw))
        assert abs(float(torch.dot(u, Aw)) - float(torch.dot(w, Au))) <= 1e-12 * scale


def test_tune_apply_sets_auto(bklib):
    """The per-order tuner of the single-order BK5 applies times both kernel
    shapes and sets KERNEL_AUTO to the faster; an AUTO apply is then bitwise
    the apply with that shape.  The process-wide table is reset afterwards."""
    from omp_bk_gb300 import tune
    bk = bklib
    orders = [(3, 300), (7, 40)]
    res = tune.tune_apply(orders, prec=bk.PREC_MIXED, layout=bk.LAYOUT_COLUMN, with_mass=True, reps=2,
                          use_cache=False)
    try:
        for p, E in orders:
            r = res[p]
            assert r["kernel"] in (bk.KERNEL_SWEEP, bk.KERNEL_COLUMN) and r["sweep_ms"] > 0 and r["column_ms"] > 0
            assert bk.bk5_auto_kernel(p, bk.PREC_MIXED, bk.LAYOUT_COLUMN, with_mass=True) == r["kernel"]
            q = p + 1
            D = bk.bk5_matrices(p)[0]
            u = bk.fill_uniform(torch.empty(E * q ** 3, dtype=torch.float32, device="cuda"), 1)
            G = bk.fill_uniform(torch.empty(6 * E * q ** 3, dtype=torch.float32, device="cuda"), 2, 0.5, 1.5)
            M = bk.fill_uniform(torch.empty(E * q ** 3, dtype=torch.float32, device="cuda"), 3, 0.5, 1.5)
            v0, v1 = torch.empty_like(u), torch.empty_like(u)
            bk.bk5_apply(p, E, D, G, u, v0, prec=bk.PREC_MIXED, layout=bk.LAYOUT_COLUMN, mass=M, lam=1.0)
            bk.bk5_apply(p, E, D, G, u, v1, prec=bk.PREC_MIXED, layout=bk.LAYOUT_COLUMN, mass=M, lam=1.0,
                         kernel=r["kernel"])
            torch.cuda.synchronize()
            assert torch.equal(v0, v1)
    finally:
        for p, _ in orders:
            bk.bk5_set_auto_kernel(p, bk.PREC_MIXED, bk.LAYOUT_COLUMN, bk.KERNEL_AUTO, with_mass=True)


def test_diagonal_matches_unit_applies(bklib, small_plan):
    """bk_hplan_diagonal against the operator itself: one unit vector per
    element (a different point in each; the element operators are
    independent), so one FP64 apply gives A_xx at all those points."""
    bk = bklib
    plan, G, M, _ = small_plan
    lam = 0.6
    diag = plan.diagonal(G, M, lam)
    u = torch.zeros(plan.n, dtype=torch.float64, device="cuda")
    idx = []
    for k, p in enumerate(plan.p):
        q3 = (p + 1) ** 3
        for e in range(plan.E[k]):
            idx.append(plan.uoff[k] + e * q3 + (7 * e + 3 * k) % q3)
    idx = torch.tensor(idx, device="cuda")
    u[idx] = 1.0
    v = torch.empty_like(u)
    plan.apply(G, M, lam, u, v, prec=bk.PREC_FP64, engine=bk.ENGINE_DFMA)
    torch.cuda.synchronize()
    got, ref = diag[idx], v[idx]
    assert float((got - ref).abs().max() / ref.abs().max()) < 1e-12
    assert bool((diag > 0).all())   # SPD: a positive diagonal


def test_cg_preconditioners(bklib, small_plan):
    """The inner CG with and without the Jacobi preconditioner: both reach
    the FP64 tolerance on the same system."""
    bk = bklib
    from omp_bk_gb300.helmholtz import PRECOND_JACOBI, PRECOND_NONE
    plan, G, M, ustar = small_plan
    f = torch.empty_like(ustar)
    plan.apply(G, M, 1.0, ustar, f, prec=bk.PREC_FP64)
    G32, M32 = G.float(), M.float()
    its = {}
    for pc in (PRECOND_NONE, PRECOND_JACOBI):
        x = torch.zeros_like(ustar)
        st = plan.cg(G, M, G32, M32, 1.0, f, x, rtol=1e-10, precond=pc)
        torch.cuda.synchronize()
        assert st["converged"] and st["relres"] <= 1e-10, (pc, st)
        assert float(torch.linalg.norm(x - ustar) / torch.linalg.norm(ustar)) < 1e-6
        its[pc] = st["inner"]
    assert its[PRECOND_JACOBI] > 0 and its[PRECOND_NONE] > 0
