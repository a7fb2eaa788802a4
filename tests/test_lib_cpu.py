"""CPU-only checks of the CUDA library: it loads, exports every function the
C headers declare, rejects bad arguments on the host (before any CUDA call),
and its 1-D rules and matrices satisfy the identities that pin them (the
reference has no such generators)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"^\s*(?:int|long long|bk_options|const char\*)\s+(bk\w+)\s*\(", src, flags=re.M))
    return names


def test_exports_every_declared_symbol(bklib):
    declared = _declared()
    assert len(declared) >= 20
    assert declared == set(bklib.EXPORTS), declared ^ set(bklib.EXPORTS)
    for name in declared:
        assert hasattr(bklib.lib(), name), name


def test_version_and_defaults(bklib):
    assert "sm_103a" in bklib.version()
    o = bklib.lib().bk_default_options()
    assert (o.prec, o.engine, o.layout, o.nfactors, o.elems_per_block) == (0, 0, 1, 6, 0)


def test_host_argument_errors(bklib):
    """with_order's 'unsupported polynomial order' and the other argument
    errors come back as status codes without a GPU."""
    L = bklib.lib()
    D = (C.c_double * 100)()
    dp = C.cast(D, C.POINTER(C.c_double))
    a16 = C.c_void_p(0x10000)
    a8 = C.c_void_p(0x10008)
    # order outside 1..8
    for p in (0, 9, -1):
        assert L.bk5_apply(p, 4, dp, a16, a16, a16, 0, None) == bklib.BK_ERR_ORDER
        assert L.bk1_apply(p, 4, dp, a16, a16, a16, 0, None) == bklib.BK_ERR_ORDER
        assert L.bk3_apply(p, 4, dp, dp, a16, a16, a16, 0, None) == bklib.BK_ERR_ORDER
    assert L.bk5_apply(3, -1, dp, a16, a16, a16, 0, None) == bklib.BK_ERR_SIZE
    assert L.bk5_apply(3, 4, dp, None, a16, a16, 0, None) == bklib.BK_ERR_NULL
    assert L.bk5_apply(3, 4, None, a16, a16, a16, 0, None) == bklib.BK_ERR_NULL
    assert L.bk5_apply(3, 4, dp, a8, a16, a16, 0, None) == bklib.BK_ERR_ALIGN
    assert L.bk1_apply(3, 4, dp, a16, a8, a16, 0, None) == bklib.BK_ERR_ALIGN
    assert L.bk3_apply(3, 4, dp, dp, a16, a16, a8, 0, None) == bklib.BK_ERR_ALIGN
    assert L.bk5_apply(3, 4, dp, a16, a16, a16, 7, None) == bklib.BK_ERR_PREC
    o = bklib.ApplyOptions(nfactors=7).c()
    assert L.bk5_apply_opt(3, 4, dp, a16, a16, a16, C.byref(o), None) == bklib.BK_ERR_PREC
    o = bklib.ApplyOptions(layout=3).c()
    assert L.bk5_apply_opt(3, 4, dp, a16, a16, a16, C.byref(o), None) == bklib.BK_ERR_PREC
    o = bklib.ApplyOptions(engine=9).c()
    assert L.bk5_apply_opt(3, 4, dp, a16, a16, a16, C.byref(o), None) == bklib.BK_ERR_PREC
    # G split into float-float pairs: the float-float engine, 6 factors, sweep kernel
    for kw in (dict(gform=2), dict(gform=bklib.G_FF, prec=bklib.PREC_MIXED),
               dict(gform=bklib.G_FF, engine=bklib.ENGINE_DFMA), dict(gform=bklib.G_FF, nfactors=9),
               dict(gform=bklib.G_FF, kernel=bklib.KERNEL_COLUMN)):
        o = bklib.ApplyOptions(**kw).c()
        assert L.bk5_apply_opt(3, 4, dp, a16, a16, a16, C.byref(o), None) == bklib.BK_ERR_PREC
    assert L.bk_g_to_ff(a16, a16, -1, None) == bklib.BK_ERR_SIZE
    assert L.bk_g_to_ff(None, a16, 4, None) == bklib.BK_ERR_NULL
    assert L.bk_g_to_ff(a16, a8, 4, None) == bklib.BK_ERR_ALIGN
    assert L.bk_g_to_ff(None, None, 0, None) == bklib.BK_OK
    # device make_bk5_G: order, factor count, layout, precision, pointers
    assert L.bk5_make_g(9, 4, a16, a16, 6, 2, 0, None) == bklib.BK_ERR_ORDER
    assert L.bk5_make_g(3, -1, a16, a16, 6, 2, 0, None) == bklib.BK_ERR_SIZE
    assert L.bk5_make_g(3, 4, a16, a16, 7, 2, 0, None) == bklib.BK_ERR_PREC
    assert L.bk5_make_g(3, 4, a16, a16, 6, 3, 0, None) == bklib.BK_ERR_PREC
    assert L.bk5_make_g(3, 4, a16, a16, 6, 2, 9, None) == bklib.BK_ERR_PREC
    assert L.bk5_make_g(3, 4, None, a16, 6, 2, 0, None) == bklib.BK_ERR_NULL
    assert L.bk5_make_g(3, 4, a16, a8, 9, 0, 0, None) == bklib.BK_ERR_ALIGN
    assert L.bk5_make_g(3, 0, None, None, 6, 2, 0, None) == bklib.BK_OK
    # BK1 qdata layouts: PQR or RQP; the device transpose_jxw
    o = bklib.ApplyOptions(jxw_layout=2).c()
    assert L.bk1_apply_opt(3, 4, dp, a16, a16, a16, C.byref(o), None) == bklib.BK_ERR_ARG
    assert L.bk1_transpose_jxw(9, 4, a16, a16, 0, None) == bklib.BK_ERR_ORDER
    assert L.bk1_transpose_jxw(3, -1, a16, a16, 0, None) == bklib.BK_ERR_SIZE
    assert L.bk1_transpose_jxw(3, 4, a16, a16, 9, None) == bklib.BK_ERR_PREC
    assert L.bk1_transpose_jxw(3, 4, None, a16, 0, None) == bklib.BK_ERR_NULL
    assert L.bk1_transpose_jxw(3, 4, a16, a8, 0, None) == bklib.BK_ERR_ALIGN
    assert L.bk1_transpose_jxw(3, 0, None, None, 0, None) == bklib.BK_OK
    # E = 0 is a no-op, even with null device pointers
    assert L.bk5_apply(3, 0, dp, None, None, None, 0, None) == bklib.BK_OK
    assert L.bk1_apply(8, 0, dp, None, None, None, 0, None) == bklib.BK_OK


def test_python_error_message(bklib):
    with pytest.raises(bklib.BKError, match="unsupported polynomial order p"):
        bklib.bk5_apply(9, 0, np.zeros(100), None, None, None)


@pytest.mark.parametrize("n", range(1, 12))
def test_gauss_rule(bklib, n):
    x, w = bklib.gauss(n)
    xr, wr = np.polynomial.legendre.leggauss(n)
    assert np.allclose(x, xr, atol=1e-15, rtol=0)
    assert np.allclose(w, wr, atol=1e-15, rtol=0)


@pytest.mark.parametrize("n", range(2, 12))
def test_gll_rule(bklib, n):
    x, w = bklib.gll(n)
    assert x[0] == -1.0 and x[-1] == 1.0
    assert np.all(np.diff(x) > 0)
    assert abs(w.sum() - 2.0) < 1e-14
    # interior points are the roots of P_{n-1}'
    dP = np.polynomial.legendre.Legendre.basis(n - 1).deriv()
    if n > 2:
        assert np.max(np.abs(dP(x[1:-1]))) < 1e-12 * max(1.0, np.max(np.abs(dP.coef)))
    # exact for polynomials of degree 2n - 3
    for deg in range(2 * n - 2):
        exact = 0.0 if deg % 2 else 2.0 / (deg + 1)
        assert abs(w @ x ** deg - exact) < 1e-13


@pytest.mark.parametrize("p", range(1, 9))
def test_interp_and_deriv_identities(bklib, p):
    B, D3, xq, wq, xn = bklib.bk1_bk3_matrices(p)
    P, Q = p + 1, p + 2
    B = B.reshape(P, Q)
    assert np.allclose(B.sum(axis=0), 1.0, atol=1e-13)        # B^T 1 = 1
    assert np.allclose(xn @ B, xq, atol=1e-13)                 # interpolates x exactly
    D3 = D3.reshape(Q, Q)                                      # D(n, q) = l_n'(x_q)
    assert np.allclose(D3.sum(axis=0), 0.0, atol=1e-12)        # derivative of 1
    assert np.allclose(xq @ D3, 1.0, atol=1e-12)               # derivative of x
    D5, x, w = bklib.bk5_matrices(p)
    D5 = D5.reshape(p + 1, p + 1)                              # D(i, n) = l_n'(x_i)
    assert np.allclose(D5.sum(axis=1), 0.0, atol=1e-12)
    assert np.allclose(D5 @ x, 1.0, atol=1e-12)
    if p >= 2:
        assert np.allclose(D5 @ x ** 2, 2 * x, atol=1e-11)


def test_auto_kernel_table(bklib):
    """BK5's KERNEL_AUTO table: the built-in rule by default, a tuned shape
    once set, the rule again after a reset; argument checks (no GPU needed)."""
    bk = bklib
    L = bk.lib()
    # the built-in rule: column kernel for FP32 storage, column layout, at
    # p <= 3 and at p = 5 with a mass term
    for p, mass, want in ((1, False, bk.KERNEL_COLUMN), (3, True, bk.KERNEL_COLUMN), (4, False, bk.KERNEL_SWEEP),
                          (4, True, bk.KERNEL_SWEEP), (5, False, bk.KERNEL_SWEEP), (5, True, bk.KERNEL_COLUMN),
                          (7, True, bk.KERNEL_SWEEP)):
        assert bk.bk5_auto_kernel(p, bk.PREC_MIXED, bk.LAYOUT_COLUMN, with_mass=mass) == want, (p, mass)
        assert bk.bk5_auto_kernel(p, bk.PREC_FP32, bk.LAYOUT_COLUMN, with_mass=mass) == want, (p, mass)
    assert bk.bk5_auto_kernel(3, bk.PREC_FP64, bk.LAYOUT_COLUMN) == bk.KERNEL_SWEEP
    assert bk.bk5_auto_kernel(3, bk.PREC_MIXED, bk.LAYOUT_INTERLEAVED) == bk.KERNEL_SWEEP
    bk.bk5_set_auto_kernel(3, bk.PREC_MIXED, bk.LAYOUT_COLUMN, bk.KERNEL_SWEEP, with_mass=True)
    assert bk.bk5_auto_kernel(3, bk.PREC_MIXED, bk.LAYOUT_COLUMN, with_mass=True) == bk.KERNEL_SWEEP
    assert bk.bk5_auto_kernel(3, bk.PREC_MIXED, bk.LAYOUT_COLUMN, with_mass=False) == bk.KERNEL_COLUMN
    bk.bk5_set_auto_kernel(3, bk.PREC_MIXED, bk.LAYOUT_COLUMN, bk.KERNEL_AUTO, with_mass=True)
    assert bk.bk5_auto_kernel(3, bk.PREC_MIXED, bk.LAYOUT_COLUMN, with_mass=True) == bk.KERNEL_COLUMN
    assert L.bk5_set_auto_kernel(9, 0, 0, 2, 0, 1) == bk.BK_ERR_ORDER
    assert L.bk5_set_auto_kernel(3, 7, 0, 2, 0, 1) == bk.BK_ERR_PREC
    assert L.bk5_set_auto_kernel(3, 0, 0, 3, 0, 1) == bk.BK_ERR_PREC
    assert L.bk5_set_auto_kernel(3, 0, 0, 2, 0, 5) == bk.BK_ERR_ARG
    assert L.bk5_auto_kernel(0, 0, 0, 2, 0) == -bk.BK_ERR_ORDER


def test_tuner_candidates():
    """The tile sizes the Helmholtz tuner tries (no GPU): for the sweep body
    the counts whose lines fill 1..SWEEPS sweeps of the block, each within
    the plan's line limit; for the column body the line budgets."""
    from omp_bk_gb300 import tune
    for p in range(2, 9):
        q2 = (p + 1) ** 2
        for block in tune.BLOCKS:
            c = tune.candidates(p, block)
            assert c == sorted(set(c)) and c
            assert all(eb >= 1 and eb * q2 <= tune.MAX_TILE_LINES for eb in c)
            assert max(1, block // q2) in c
            full = [max(1, k * block // q2) for k in range(1, tune.SWEEPS + 1)
                    if max(1, k * block // q2) * q2 <= tune.MAX_TILE_LINES]
            assert set(full) == set(c)
        assert tune.candidates(p) == sorted({tune.tiles_for(p, t) for t in tune.LINE_BUDGETS})
