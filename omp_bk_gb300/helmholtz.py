"""Batched mixed-order Helmholtz operator A = K + lambda M (BK5 Laplacian K,
collocated GLL mass M) and its mixed-precision CG solver, over the C ABI of
include/bk_solver.h.

Elements of each order p are stored one order after another (u, v, mass:
E_p (p+1)^3 values; G: E_p 6 (p+1)^3 values in the column layout).  One
persistent launch applies the operator to all orders; the solver's inner
FP32 CG runs as one CUDA graph (conditional WHILE node) per refinement step.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import (BK_OK, BKError, ENGINE_AUTO, LAYOUT_COLUMN, PREC_FP64, PREC_MIXED, _ptr, _stream, bk5_matrices,
               check, geom_trilinear, lib)

BK_ERR_NOCONV = 9


class OrderRange(C.Structure):
    _fields_ = [("p", C.c_int), ("E", C.c_int64), ("elems_per_tile", C.c_int)]


PRECOND_NONE, PRECOND_JACOBI = 0, 1


class CGOptions(C.Structure):
    _fields_ = [("rtol", C.c_double), ("max_outer", C.c_int), ("inner_rtol", C.c_double), ("max_inner", C.c_int),
                ("precond", C.c_int)]


class CGStats(C.Structure):
    _fields_ = [("outer", C.c_int), ("inner", C.c_int), ("relres", C.c_double)]


def _declare():
    L = lib()
    if getattr(L, "_hplan_declared", False):
        return L
    L.bk_hplan_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.POINTER(OrderRange),
                                  C.POINTER(C.POINTER(C.c_double)), C.c_void_p]
    L.bk_hplan_destroy.argtypes = [C.c_void_p]
    L.bk_hplan_size.argtypes = [C.c_void_p, C.c_int]
    L.bk_hplan_size.restype = C.c_longlong
    L.bk_hplan_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_int,
                                 C.c_int, C.c_void_p]
    L.bk_hplan_cg.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                              C.c_void_p, C.POINTER(CGOptions), C.POINTER(CGStats), C.c_void_p]
    L.bk_hplan_set_kernel.argtypes = [C.c_void_p, C.c_int]
    L.bk_hplan_diagonal.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]
    L.bk_hplan_diagonal.restype = C.c_int
    L.bk_hplan_set_shape.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.bk_hplan_set_fp64_shape.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_int, C.c_void_p]
    for f in ("bk_hplan_create", "bk_hplan_destroy", "bk_hplan_apply", "bk_hplan_cg", "bk_hplan_set_kernel",
              "bk_hplan_set_shape", "bk_hplan_set_fp64_shape"):
        getattr(L, f).restype = C.c_int
    L._hplan_declared = True
    return L


def default_tiles(p: int) -> int:
    """Elements per tile when no tuning is given (the library's own default):
    about 128 lines of (p+1) points, at least one element."""
    q2 = (p + 1) ** 2
    return 1 if q2 >= 100 else (2 if q2 >= 64 else (128 + q2 - 1) // q2)


class HelmholtzPlan:
    """orders: list of (p, E) or (p, E, elems_per_tile)."""

    def __init__(self, orders, stream=None, block=0, gstage=0):
        L = _declare()
        self.orders = [tuple(o) + (0,) * (3 - len(o)) for o in orders]
        self.p = [o[0] for o in self.orders]
        self.E = [int(o[1]) for o in self.orders]
        arr = (OrderRange * len(self.orders))(*[OrderRange(p, E, eb) for p, E, eb in self.orders])
        self._D = [np.ascontiguousarray(bk5_matrices(p)[0]) for p in self.p]
        dptr = (C.POINTER(C.c_double) * len(self._D))(*[d.ctypes.data_as(C.POINTER(C.c_double)) for d in self._D])
        h = C.c_void_p()
        check(L.bk_hplan_create(C.byref(h), len(self.orders), arr, dptr, _stream(stream)), "bk_hplan_create")
        self.h = h
        if block or gstage:
            self.set_shape(block, gstage)
        self.n = L.bk_hplan_size(h, 0)
        self.ng = L.bk_hplan_size(h, 1)
        self.ntiles = L.bk_hplan_size(h, 2)
        # offsets of each order in u and G
        self.uoff, self.goff = [], []
        uo = go = 0
        for p, E in zip(self.p, self.E):
            self.uoff.append(uo)
            self.goff.append(go)
            uo += E * (p + 1) ** 3
            go += 6 * E * (p + 1) ** 3

    @property
    def kernel(self) -> int:
        """The body of the persistent launch: KERNEL_SWEEP (even-odd line
        sweeps) or KERNEL_COLUMN."""
        return int(_declare().bk_hplan_size(self.h, 3))

    def set_shape(self, block: int = 0, gstage: int = 0):
        """Threads per block of the sweep body's launch (0: the largest
        tile's lines; tiles with more lines loop over them) and, for FP32
        storage, whether G is staged in shared memory (bk_hplan_set_shape)."""
        check(_declare().bk_hplan_set_shape(self.h, int(block), int(gstage)), "bk_hplan_set_shape")

    def set_fp64_shape(self, tiles=None, block: int = 0, stream=None):
        """Tiles and threads of the FP64-storage launches apart from the FP32
        ones (bk_hplan_set_fp64_shape): tiles {p: elements per tile} or a list
        per range (0 keeps the range's own); None returns them to the plan's."""
        if tiles is None:
            arr = None
        else:
            eb = [int(tiles.get(p, 0)) for p in self.p] if isinstance(tiles, dict) else [int(t) for t in tiles]
            if len(eb) != len(self.p):
                raise ValueError("one tile size per range")
            arr = (C.c_int * len(eb))(*eb)
        check(_declare().bk_hplan_set_fp64_shape(self.h, arr, int(block), _stream(stream)),
              "bk_hplan_set_fp64_shape")

    @property
    def block(self) -> int:
        return int(_declare().bk_hplan_size(self.h, 6))

    @property
    def fp64_block(self) -> int:
        """Threads (per direction group) of the FP64-storage launches."""
        return int(_declare().bk_hplan_size(self.h, 9))

    @property
    def fp64_ntiles(self) -> int:
        return int(_declare().bk_hplan_size(self.h, 8))

    @property
    def gstage(self) -> int:
        return int(_declare().bk_hplan_size(self.h, 7))

    def smem_bytes(self, fp64: bool = False) -> int:
        """Shared memory per block of the sweep body's launch for FP64
        (fp64) or FP32 storage."""
        return int(_declare().bk_hplan_size(self.h, 4 if fp64 else 5))

    def set_kernel(self, kernel: int):
        check(_declare().bk_hplan_set_kernel(self.h, int(kernel)), "bk_hplan_set_kernel")

    def close(self):
        if self.h:
            lib().bk_hplan_destroy(self.h)
            self.h = None

    __del__ = close

    def apply(self, G, mass, lam, u, v, prec=PREC_MIXED, engine=ENGINE_AUTO, stream=None):
        check(_declare().bk_hplan_apply(self.h, _ptr(G), _ptr(mass), float(lam), _ptr(u), _ptr(v), prec, engine,
                                        _stream(stream)), "bk_hplan_apply")

    def diagonal(self, G, mass, lam, out=None, stream=None):
        """diag(K + lam M) at every point (FP64 G and mass)."""
        import torch
        if out is None:
            out = torch.empty(self.n, dtype=torch.float64, device="cuda")
        check(_declare().bk_hplan_diagonal(self.h, _ptr(G), _ptr(mass), float(lam), _ptr(out), _stream(stream)),
              "bk_hplan_diagonal")
        return out

    def cg(self, G64, mass64, G32, mass32, lam, f, x, rtol=1e-10, max_outer=8, inner_rtol=1e-5, max_inner=10000,
           stream=None, allow_noconv=False, precond=PRECOND_JACOBI):
        o = CGOptions(rtol, max_outer, inner_rtol, max_inner, precond)
        st = CGStats()
        rc = _declare().bk_hplan_cg(self.h, _ptr(G64), _ptr(mass64), _ptr(G32), _ptr(mass32), float(lam), _ptr(f),
                                    _ptr(x), C.byref(o), C.byref(st), _stream(stream))
        if rc != BK_OK and not (allow_noconv and rc == BK_ERR_NOCONV):
            raise BKError(rc, "bk_hplan_cg")
        return {"outer": st.outer, "inner": st.inner, "relres": st.relres, "converged": rc == BK_OK}

    def geometry(self, seed=7, h=1.0, jitter=0.15, stream=None):
        """G (column layout) and the collocated mass of every order, in FP64:
        each order its own jittered trilinear mesh of unit-size elements
        (spacing h)."""
        import torch
        G = torch.empty(self.ng, dtype=torch.float64, device="cuda")
        M = torch.empty(self.n, dtype=torch.float64, device="cuda")
        for k, (p, E) in enumerate(zip(self.p, self.E)):
            q = p + 1
            _, x, w = bk5_matrices(p)
            nx = 1 << max(0, math.ceil(math.log2(max(1.0, E ** (1.0 / 3.0)) - 1e-9)))
            if E == 0:
                continue
            geom_trilinear(q, E, nx, nx, x, w, seed + p, h, jitter,
                           G=G[self.goff[k]: self.goff[k] + 6 * E * q ** 3], layout=LAYOUT_COLUMN,
                           mass=M[self.uoff[k]: self.uoff[k] + E * q ** 3], stream=stream)
        return G, M


def config_orders():
    """The mixed-order configuration: p = 2..8, E_p = 2^(8-p) 4096 elements
    (43,536,384 DoFs)."""
    return [(p, (2 ** (8 - p)) * 4096) for p in range(2, 9)]
