"""CPU oracle of the bake-off operator apply -- TEST INFRASTRUCTURE.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package: it is the checker of the CUDA kernels, never
the thing measured or shipped.  The ``omp_bk_gb300`` package does not import
it and has no CPU fallback.

``liboracle.so`` (``bk_oracle.c``) restates the reference's host kernels and
harness references in plain C; ``_ref/libbkref_*.so`` are the reference's own
kernels compiled from its sources (only where those sources are present).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_libs: dict = {}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_sz = C.c_size_t


def build(ref: bool = False) -> None:
    """Compile liboracle.so / liboracle_fast.so (and the reference's own
    kernels under _ref/ when ``ref`` and its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _declare(lib, name, restype, argtypes):
    f = getattr(lib, name)
    f.restype = restype
    f.argtypes = argtypes


def lib(fast: bool = False):
    """The oracle library (``fast``: the -O3, FP-contracting build used as the
    CPU baseline; otherwise the checker build without contraction)."""
    key = "fast" if fast else "check"
    if key in _libs:
        return _libs[key]
    path = os.path.join(HERE, "liboracle_fast.so" if fast else "liboracle.so")
    if not os.path.exists(path):
        build()
    L = C.CDLL(path)
    for sfx, p in (("", _dp), ("_f32", _fp)):
        _declare(L, "bko_bk1_sumfact" + sfx, None, [C.c_int, _sz, p, p, p, p])
        _declare(L, "bko_bk3_sumfact" + sfx, None, [C.c_int, _sz, p, p, p, p, p])
        _declare(L, "bko_bk3_sumfact_k" + sfx, None, [C.c_int, _sz, p, p, p, C.c_void_p, p, p])
        _declare(L, "bko_bk5_sumfact" + sfx, None, [C.c_int, _sz, p, p, p, p])
        _declare(L, "bko_bk5_sumfact_h" + sfx, None,
                 [C.c_int, _sz, p, p, C.c_void_p, C.c_double if sfx == "" else C.c_float, p, p])
    _declare(L, "bko_reference_bk1", None, [C.c_int, _sz, _fp, _fp, _fp, _dp])
    _declare(L, "bko_reference_bk3", None, [C.c_int, _sz, _fp, _fp, _fp, _fp, _dp])
    _declare(L, "bko_reference_bk5", None, [C.c_int, _sz, _fp, _fp, _fp, _dp])
    _declare(L, "bko_make_bk5_G", None, [_dp, _sz, C.c_int, C.c_int, C.c_int, _dp])
    _declare(L, "bko_transpose_jxw", None, [_dp, _sz, C.c_int, _dp])
    _declare(L, "bko_make_test_basis", None, [C.c_int, C.c_int, _dp])
    _declare(L, "bko_make_test_basis_f32", None, [C.c_int, C.c_int, _fp])
    _declare(L, "bko_fill_random_test_data", None, [_dp, _sz, _dp, _sz, C.c_uint32])
    _declare(L, "bko_norm2", C.c_double, [_dp, _sz])
    _declare(L, "bko_norm2_f32", C.c_double, [_fp, _sz])
    _declare(L, "bko_rel_maxdiff", C.c_double, [_dp, _dp, _sz])
    _declare(L, "bko_bk3_adjoint", None, [C.c_int, _sz, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp])
    _declare(L, "bko_max_nq", C.c_int, [])
    # inputs of the benchmark configurations (bk_geom_oracle.c)
    u64 = C.c_uint64
    _declare(L, "bko_splitmix64", u64, [u64])
    _declare(L, "bko_uniform01", C.c_double, [u64, u64])
    _declare(L, "bko_fill_uniform", None, [_dp, _sz, u64, C.c_double, C.c_double])
    _declare(L, "bko_fill_lognormal", None, [_dp, _sz, u64, C.c_double])
    _declare(L, "bko_gauss", C.c_int, [C.c_int, _dp, _dp])
    _declare(L, "bko_gll", C.c_int, [C.c_int, _dp, _dp])
    _declare(L, "bko_lagrange_interp", C.c_int, [C.c_int, _dp, C.c_int, _dp, _dp])
    _declare(L, "bko_lagrange_deriv", C.c_int, [C.c_int, _dp, _dp])
    _declare(L, "bko_geom_affine", None, [C.c_int, _sz, _sz, _dp, _dp, u64, C.c_double, C.c_double,
                                          C.c_void_p, C.c_void_p, C.c_int])
    _declare(L, "bko_coords_affine", None, [C.c_int, _sz, _sz, C.c_int, C.c_int, _dp, u64, C.c_double,
                                            C.c_double, _dp])
    _declare(L, "bko_geom_trilinear", None, [C.c_int, _sz, _sz, C.c_int, C.c_int, _dp, _dp, u64, C.c_double,
                                             C.c_double, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p])
    _libs[key] = L
    return L


# ---- numpy-level helpers ----------------------------------------------------

def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _real(a):
    return np.float32 if np.asarray(a).dtype == np.float32 else np.float64


def bk1(nq, E, basis, jxw, u, fast=False):
    """openmp/bk1_sumfact.h:17-159 restated: v = B^T diag(JxW) B u per element."""
    dt = _real(u)
    out = np.empty(E * (nq - 1) ** 3, dtype=dt)
    f = lib(fast).bko_bk1_sumfact_f32 if dt == np.float32 else lib(fast).bko_bk1_sumfact
    f(nq, E, _c(basis, dt), _c(jxw, dt), _c(u, dt), out)
    return out


def bk3(nq, E, basis, dbasis, G, u, k=None, fast=False):
    """openmp/bk3_sumfact.h:18-187 restated (k: optional coefficient at the
    quadrature points, no reference counterpart)."""
    dt = _real(u)
    out = np.empty(E * (nq - 1) ** 3, dtype=dt)
    L = lib(fast)
    f = L.bko_bk3_sumfact_k_f32 if dt == np.float32 else L.bko_bk3_sumfact_k
    kk = None if k is None else _c(k, dt)
    f(nq, E, _c(basis, dt), _c(dbasis, dt), _c(G, dt),
      None if kk is None else kk.ctypes.data_as(C.c_void_p), _c(u, dt), out)
    return out


def bk5(nq, E, dbasis, G, u, mass=None, lam=0.0, fast=False):
    """openmp/BK5.cpp:19-103 restated (mass: optional diagonal Helmholtz term
    lam * mass * u, no reference counterpart)."""
    dt = _real(u)
    out = np.empty(E * nq ** 3, dtype=dt)
    L = lib(fast)
    f = L.bko_bk5_sumfact_h_f32 if dt == np.float32 else L.bko_bk5_sumfact_h
    m = None if mass is None else _c(mass, dt)
    f(nq, E, _c(dbasis, dt), _c(G, dt), None if m is None else m.ctypes.data_as(C.c_void_p),
      lam, _c(u, dt), out)
    return out


def bk3_adjoint(nq, E, basis, dbasis, G, k, u, res):
    """dL/dk and dL/dG of L = 1/2 |A(k) u - f|^2 given res = A(k) u - f."""
    d = np.float64
    dk = np.empty(E * nq ** 3, dtype=d)
    dG = np.empty(E * 6 * nq ** 3, dtype=d)
    lib().bko_bk3_adjoint(nq, E, _c(basis, d), _c(dbasis, d), _c(G, d), _c(k, d), _c(u, d),
                          _c(res, d), dk, dG)
    return dk, dG


def make_bk5_G(G6i, E, nq, F, layout):
    out = np.empty(E * F * nq ** 3, dtype=np.float64)
    lib().bko_make_bk5_G(_c(G6i, np.float64), E, nq, F, layout, out)
    return out


def transpose_jxw(jxw, E, nq):
    out = np.empty(E * nq ** 3, dtype=np.float64)
    lib().bko_transpose_jxw(_c(jxw, np.float64), E, nq, out)
    return out


def test_basis(rows, cols, dtype=np.float64):
    m = np.empty(rows * cols, dtype=dtype)
    if dtype == np.float32:
        lib().bko_make_test_basis_f32(rows, cols, m)
    else:
        lib().bko_make_test_basis(rows, cols, m)
    return m


def random_test_data(nin, njxw, seed=12345):
    a = np.empty(nin, dtype=np.float64)
    b = np.empty(njxw, dtype=np.float64)
    lib().bko_fill_random_test_data(a, nin, b, njxw, seed)
    return a, b


def norm2(v):
    v = np.ascontiguousarray(v)
    if v.dtype == np.float32:
        return lib().bko_norm2_f32(v, v.size)
    return lib().bko_norm2(_c(v, np.float64), v.size)


def rel_maxdiff(out, ref):
    out = _c(out, np.float64)
    ref = _c(ref, np.float64)
    return lib().bko_rel_maxdiff(out, ref, out.size)


def reference_bk1(nq, E, basis, jxw, u):
    out = np.empty(E * (nq - 1) ** 3)
    f = np.float32
    lib().bko_reference_bk1(nq, E, _c(basis, f), _c(jxw, f), _c(u, f), out)
    return out


def reference_bk3(nq, E, basis, D, G, u):
    out = np.empty(E * (nq - 1) ** 3)
    f = np.float32
    lib().bko_reference_bk3(nq, E, _c(basis, f), _c(D, f), _c(G, f), _c(u, f), out)
    return out


def reference_bk5(nq, E, D, G6i, u):
    out = np.empty(E * nq ** 3)
    f = np.float32
    lib().bko_reference_bk5(nq, E, _c(D, f), _c(G6i, f), _c(u, f), out)
    return out


# ---- inputs of the benchmark configurations (bk_geom_oracle.c) ----------------

def _opt(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def uniform(n, seed, lo=-1.0, hi=1.0, fast=False):
    """lo + (hi - lo) U(seed, i), i = 0..n-1 (splitmix64 streams)."""
    out = np.empty(int(n))
    lib(fast).bko_fill_uniform(out, out.size, seed, lo, hi)
    return out


def lognormal(n, seed, sigma, fast=False):
    out = np.empty(int(n))
    lib(fast).bko_fill_lognormal(out, out.size, seed, sigma)
    return out


def gauss(n):
    x, w = np.empty(n), np.empty(n)
    assert lib().bko_gauss(n, x, w) == 0
    return x, w


def gll(n):
    x, w = np.empty(n), np.empty(n)
    assert lib().bko_gll(n, x, w) == 0
    return x, w


def lagrange_interp(nodes, pts):
    nodes, pts = _c(nodes, np.float64), _c(pts, np.float64)
    B = np.empty(nodes.size * pts.size)
    assert lib().bko_lagrange_interp(nodes.size, nodes, pts.size, pts, B) == 0
    return B


def lagrange_deriv(x):
    x = _c(x, np.float64)
    D = np.empty(x.size * x.size)
    assert lib().bko_lagrange_deriv(x.size, x, D) == 0
    return D


def bk5_matrices(p):
    """(D, x, w) of BK5 at order p: Q = p + 1 GLL points, D(i, n) = l_n'(x_i)
    (openmp/BK5.cpp's dbasis[i*nq + n])."""
    x, w = gll(p + 1)
    return lagrange_deriv(x), x, w


def bk1_bk3_matrices(p):
    """(B, D, gauss x, gauss w, gll x) of BK1/BK3 at order p: B(i, q) =
    l_i(xq_q) from P = p + 1 GLL nodes to Q = p + 2 Gauss points, and BK3's
    D(n, q) = l_n'(xq_q) on the Gauss points (openmp/bk3_sumfact.h's
    dbasis[n*nq + q])."""
    xn, _ = gll(p + 1)
    xq, wq = gauss(p + 2)
    B = lagrange_interp(xn, xq)
    Q = p + 2
    D = lagrange_deriv(xq).reshape(Q, Q).T.copy().ravel()
    return B, D, xq, wq, xn


def geom_affine(Q, e0, ne, x, w, seed, h, pert, qdata=True, G=True, layout=0, fast=False):
    """(qdata, G) of elements e0..e0+ne-1 of the affine mesh (None where not
    asked for)."""
    Q3 = Q ** 3
    q = np.empty(ne * Q3) if qdata else None
    g = np.empty(ne * 6 * Q3) if G else None
    lib(fast).bko_geom_affine(Q, e0, ne, _c(x, np.float64), _c(w, np.float64), seed, h, pert, _opt(q), _opt(g),
                              layout)
    return q, g


def coords_affine(Q, e0, ne, nx, ny, x, seed, h, pert):
    out = np.empty(ne * Q ** 3 * 3)
    lib().bko_coords_affine(Q, e0, ne, nx, ny, _c(x, np.float64), seed, h, pert, out)
    return out


def geom_trilinear(Q, e0, ne, nx, ny, x, w, seed, h, jit, G=True, layout=1, mass=False, coords=False,
                   fast=False):
    """(G, mass, coords) of elements e0..e0+ne-1 of the jittered trilinear
    mesh on an nx x ny x .. grid (None where not asked for)."""
    Q3 = Q ** 3
    g = np.empty(ne * 6 * Q3) if G else None
    m = np.empty(ne * Q3) if mass else None
    c = np.empty(ne * Q3 * 3) if coords else None
    lib(fast).bko_geom_trilinear(Q, e0, ne, nx, ny, _c(x, np.float64), _c(w, np.float64), seed, h, jit, _opt(g),
                                 layout, _opt(m), _opt(c))
    return g, m, c
