"""The GPU input generators (omp_bk_gb300/csrc/bk_geom.cu) held to the
oracle's FP64 host restatement (oracle/bk_geom_oracle.c), which forms J^-1 by
cross products of J's columns instead of the GPU's per-point cofactors: the
seeded fields, the affine and jittered-trilinear meshes' qdata, G (every
layout), collocated mass and coordinates, on the first elements of each
benchmark configuration's own seed and sizes, plus an analytic case.

Tolerance: max |gpu - oracle| / max |oracle| <= 1e-14 per array (the two
formulas agree to rounding, not bit for bit)."""
import math

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-14
NE = 300   # elements compared per case


def _rel(a, ref):
    a, ref = np.asarray(a, dtype=np.float64), np.asarray(ref, dtype=np.float64)
    return float(np.abs(a - ref).max() / np.abs(ref).max())


def _z(n):
    return torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")


def _host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def test_fields(bklib):
    """U[-1,1] (seeds of u, f and the FD directions) and log-normal k."""
    for seed, lo, hi in ((1, -1.0, 1.0), (22, -1.0, 1.0), (44, -1.0, 1.0), (1003, 0.5, 1.5)):
        g = bklib.fill_uniform(_z(100003), seed, lo, hi)
        ref = oracle.uniform(100003, seed, lo, hi)
        assert np.abs(_host(g) - ref).max() <= 2 * np.finfo(np.float64).eps * max(abs(lo), abs(hi))
    g32 = bklib.fill_uniform(torch.empty(4097, dtype=torch.float32, device="cuda"), 7)
    assert np.array_equal(_host(g32), oracle.uniform(4097, 7).astype(np.float32))
    k = bklib.fill_lognormal(_z(65536), 42, 0.5)
    assert _rel(_host(k), oracle.lognormal(65536, 42, 0.5)) <= TOL


@pytest.mark.parametrize("name,p,seed,h,pert,layout", [
    ("bk1 p=3", 3, 21, 1.0 / 16, 0.2, 0),
    ("bk3 p=6", 6, 31, 1.0 / 64, 0.2, 0),
    ("adjoint p=4", 4, 41, 1.0 / 16, 0.2, 0),
    ("bk3 p=6 interleaved", 6, 31, 1.0 / 64, 0.2, 1),
    ("bk3 p=6 column", 6, 31, 1.0 / 64, 0.2, 2),
])
def test_affine(bklib, name, p, seed, h, pert, layout):
    """BK1/BK3 and the adjoint: Gauss points Q = p + 2, affine elements."""
    B, D, xq, wq, xn = bklib.bk1_bk3_matrices(p)
    Q = p + 2
    qd, G = _z(NE * Q ** 3), _z(NE * 6 * Q ** 3)
    bklib.geom_affine(Q, NE, xq, wq, seed, h, pert, qdata=qd, G=G, layout=layout)
    rq, rG = oracle.geom_affine(Q, 0, NE, xq, wq, seed, h, pert, layout=layout)
    assert _rel(_host(qd), rq) <= TOL, name
    assert _rel(_host(G), rG) <= TOL, name
    # the six factors separately (off-diagonal factors are ~pert of the diagonal)
    gg, rr = _host(G).reshape(NE, -1), rG.reshape(NE, -1)
    assert np.abs(gg - rr).max() <= TOL * np.abs(rr).max()
    if name.startswith("bk3 p=6") and layout == 0:
        # the nodes' coordinates (the smooth input sin(pi x) sin(pi y) sin(pi z))
        P = p + 1
        X = _z(NE * P ** 3 * 3)
        bklib.coords_affine(P, NE, 64, 64, xn, seed, h, pert, X)
        assert _rel(_host(X), oracle.coords_affine(P, 0, NE, 64, 64, xn, seed, h, pert)) <= TOL


def test_affine_analytic(bklib):
    """pert = 0: G = w (h/2) I and qdata = w h^3 / 8 (sum h^3 per element)."""
    p, h = 4, 1.0 / 16
    _, _, xq, wq, _ = bklib.bk1_bk3_matrices(p)
    Q, E = p + 2, 4
    qd, G = _z(E * Q ** 3), _z(E * 6 * Q ** 3)
    bklib.geom_affine(Q, E, xq, wq, 3, h, 0.0, qdata=qd, G=G, layout=0)
    W = np.einsum("i,j,k->ijk", wq, wq, wq).ravel()
    q = _host(qd).reshape(E, -1)
    assert np.abs(q.sum(axis=1) - h ** 3).max() <= 1e-15
    g = _host(G).reshape(E, 6, -1)
    for f, diag in enumerate((1, 0, 0, 1, 0, 1)):
        assert np.abs(g[:, f] - diag * W * h / 2).max() <= 1e-16


@pytest.mark.parametrize("nx,layout", [(64, 2), (64, 1), (64, 0), (4, 2)])
def test_trilinear_bk5(bklib, nx, layout):
    """The headline's mesh: GLL p = 7, a 64 x 64 x .. grid of spacing 1/64,
    vertex jitter 0.15 h, seed 2 (nx = 4: elements in several grid layers);
    G, the collocated mass and the coordinates."""
    p, h, jit, seed = 7, 1.0 / 64, 0.15, 2
    D, x, w = bklib.bk5_matrices(p)
    Q = p + 1
    G, M, X = _z(NE * 6 * Q ** 3), _z(NE * Q ** 3), _z(NE * Q ** 3 * 3)
    bklib.geom_trilinear(Q, NE, nx, nx, x, w, seed, h, jit, G=G, layout=layout, mass=M, coords=X)
    rG, rM, rX = oracle.geom_trilinear(Q, 0, NE, nx, nx, x, w, seed, h, jit, layout=layout, mass=True,
                                       coords=True)
    assert _rel(_host(G), rG) <= TOL
    assert _rel(_host(M), rM) <= TOL
    assert _rel(_host(X), rX) <= TOL


@pytest.mark.parametrize("p", [2, 5, 8])
def test_trilinear_helmholtz(bklib, p):
    """The mixed-order Helmholtz plan's per-order meshes (unit elements,
    seed 11 + p, grid side the power of two above E_p^(1/3))."""
    from omp_bk_gb300 import helmholtz as hz
    E = 96
    plan = hz.HelmholtzPlan([(p, E)])
    try:
        G, M = plan.geometry(seed=11)
    finally:
        plan.close()
    _, x, w = bklib.bk5_matrices(p)
    nx = 1 << max(0, math.ceil(math.log2(max(1.0, E ** (1.0 / 3.0)) - 1e-9)))
    rG, rM, _ = oracle.geom_trilinear(p + 1, 0, E, nx, nx, x, w, 11 + p, 1.0, 0.15, layout=2, mass=True)
    assert _rel(_host(G), rG) <= TOL
    assert _rel(_host(M), rM) <= TOL
