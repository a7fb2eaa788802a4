"""omp_bk_gb300 -- GB300 (sm_103a) bake-off operator apply: BK1 mass, BK3
Poisson, BK5 collocated Laplacian on element-major hexahedral E-vectors.

The compute path is the CUDA library ``_lib/libbk_gb300.so`` behind the C ABI
of ``include/bk_gpu.h`` (built by ``omp_bk_gb300.build``).  This module is a
thin ctypes layer over it, mirroring the reference's operator interface
``bk::SumFactorization<T, nq>(nelmt, basis, JxW|G, in, out)``
(openmp/bk1_sumfact.h:16-22, openmp/bk3_sumfact.h:17-24, openmp/BK5.cpp:18-24):
the same argument order and meaning, the order p dispatched at run time as
``bk::with_order`` does (include/bk_common.h:148-178), and an unsupported
order reported as ``unsupported polynomial order p = <p>``.  Device arrays are
torch CUDA tensors (torch is used for device memory and streams only).

There is no CPU fallback: without the built library every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_lib", "libbk_gb300.so")

# status codes (bk_gpu.h)
BK_OK, BK_ERR_ORDER, BK_ERR_SIZE, BK_ERR_ALIGN, BK_ERR_NULL, BK_ERR_PREC, BK_ERR_CUDA, BK_ERR_TIMEOUT, BK_ERR_ARG = range(9)
STATUS_NAMES = {0: "ok", 1: "unsupported polynomial order p", 2: "bad element count", 3: "misaligned pointer",
                4: "null pointer", 5: "unsupported precision/engine/layout", 6: "CUDA error",
                7: "device wait timed out", 8: "invalid argument"}
# precisions, engines, layouts
PREC_FP64, PREC_FP32, PREC_MIXED = 0, 1, 2
ENGINE_AUTO, ENGINE_DFMA, ENGINE_FF = 0, 1, 2
LAYOUT_FACTOR, LAYOUT_INTERLEAVED, LAYOUT_COLUMN = 0, 1, 2
KERNEL_AUTO, KERNEL_SWEEP, KERNEL_COLUMN = 0, 1, 2
G_STORAGE, G_FF = 0, 1
JXW_PQR, JXW_RQP = 0, 1

# every symbol the C headers declare (checked by the CPU tests)
EXPORTS = [
    "bk_default_options", "bk1_apply", "bk3_apply", "bk5_apply", "bk1_apply_opt", "bk3_apply_opt",
    "bk5_apply_opt", "bk5_apply_ex", "bk3_apply_k", "bk_device_status", "bk_set_wait_limit",
    "bk_test_wait_timeout", "bk_version",
    "bk_gauss_points", "bk_gll_points", "bk_lagrange_interp", "bk_lagrange_deriv", "bk_fill_uniform",
    "bk_fill_lognormal", "bk_geom_affine", "bk_coords_affine", "bk_geom_trilinear", "bk_convert",
    "bk3_adjoint", "bk_stream_kernel", "bk_dot_workspace_bytes", "bk_dot", "bk_axpby",
    "bk_hplan_create", "bk_hplan_destroy", "bk_hplan_size", "bk_hplan_set_kernel", "bk_hplan_set_shape",
    "bk_hplan_set_fp64_shape",
    "bk_hplan_apply", "bk_hplan_cg", "bk_hplan_diagonal",
    "bk_dot_noalloc",
    "bk_host_plan_create", "bk_host_plan_destroy", "bk1_apply_host", "bk3_apply_host", "bk5_apply_host",
    "bk_g_to_ff", "bk5_make_g", "bk1_transpose_jxw", "bk_probe_contract", "bk5_set_auto_kernel",
    "bk5_auto_kernel",
]


class BKError(RuntimeError):
    """A non-zero status of the C ABI."""

    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"{what}: {STATUS_NAMES.get(code, 'error')} (status {code})")


class Options(C.Structure):
    _fields_ = [("prec", C.c_int), ("engine", C.c_int), ("layout", C.c_int), ("nfactors", C.c_int),
                ("elems_per_block", C.c_int), ("kernel", C.c_int), ("gform", C.c_int), ("jxw_layout", C.c_int)]


_lib = None
_vp = C.c_void_p
_dp = C.POINTER(C.c_double)
_i64 = C.c_int64


def lib():
    """The loaded CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m omp_bk_gb300.build` "
                           "(there is no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    sig = {
        "bk1_apply": [C.c_int, _i64, _dp, _vp, _vp, _vp, C.c_int, _vp],
        "bk3_apply": [C.c_int, _i64, _dp, _dp, _vp, _vp, _vp, C.c_int, _vp],
        "bk5_apply": [C.c_int, _i64, _dp, _vp, _vp, _vp, C.c_int, _vp],
        "bk1_apply_opt": [C.c_int, _i64, _dp, _vp, _vp, _vp, C.POINTER(Options), _vp],
        "bk3_apply_opt": [C.c_int, _i64, _dp, _dp, _vp, _vp, _vp, C.POINTER(Options), _vp],
        "bk5_apply_opt": [C.c_int, _i64, _dp, _vp, _vp, _vp, C.POINTER(Options), _vp],
        "bk5_apply_ex": [C.c_int, _i64, _dp, _vp, _vp, _vp, C.c_double, _vp, C.POINTER(Options), _vp],
        "bk3_apply_k": [C.c_int, _i64, _dp, _dp, _vp, _vp, _vp, _vp, C.POINTER(Options), _vp],
        "bk_device_status": [C.POINTER(C.c_int), C.c_int, _vp],
        "bk_set_wait_limit": [C.c_longlong],
        "bk_test_wait_timeout": [_vp],
        "bk_gauss_points": [C.c_int, _dp, _dp],
        "bk_gll_points": [C.c_int, _dp, _dp],
        "bk_lagrange_interp": [C.c_int, _dp, C.c_int, _dp, _dp],
        "bk_lagrange_deriv": [C.c_int, _dp, _dp],
        "bk_fill_uniform": [_vp, C.c_longlong, C.c_ulonglong, C.c_double, C.c_double, C.c_int, _vp],
        "bk_fill_lognormal": [_vp, C.c_longlong, C.c_ulonglong, C.c_double, C.c_int, _vp],
        "bk_geom_affine": [C.c_int, C.c_longlong, _dp, _dp, C.c_ulonglong, C.c_double, C.c_double, _vp, _vp,
                           C.c_int, _vp],
        "bk_coords_affine": [C.c_int, C.c_longlong, C.c_int, C.c_int, _dp, C.c_ulonglong, C.c_double,
                             C.c_double, _vp, _vp],
        "bk_geom_trilinear": [C.c_int, C.c_longlong, C.c_int, C.c_int, _dp, _dp, C.c_ulonglong, C.c_double,
                              C.c_double, _vp, C.c_int, _vp, _vp, _vp],
        "bk_convert": [_vp, _vp, C.c_longlong, C.c_int, _vp],
        "bk3_adjoint": [C.c_int, _i64, _dp, _dp, _vp, _vp, _vp, _vp, _vp, _vp, C.POINTER(Options), _vp],
        "bk_stream_kernel": [C.c_int, C.c_longlong, _vp, _vp, _vp, C.c_int, _vp],
        "bk_dot": [C.c_longlong, _vp, _vp, C.c_int, _vp, _vp, C.c_longlong, C.c_int, _vp],
        "bk_axpby": [C.c_longlong, C.c_double, _vp, C.c_double, _vp, C.c_int, _vp],
        "bk_g_to_ff": [_vp, _vp, _i64, _vp],
        "bk5_make_g": [C.c_int, _i64, _vp, _vp, C.c_int, C.c_int, C.c_int, _vp],
        "bk1_transpose_jxw": [C.c_int, _i64, _vp, _vp, C.c_int, _vp],
        "bk_probe_contract": [C.c_int, C.c_longlong, _dp, _vp, _vp, _vp],
        "bk5_set_auto_kernel": [C.c_int] * 6,
        "bk5_auto_kernel": [C.c_int] * 5,
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.bk_dot_workspace_bytes.argtypes = [C.c_longlong]
    L.bk_dot_workspace_bytes.restype = C.c_longlong
    L.bk_version.restype = C.c_char_p
    L.bk_default_options.restype = Options
    _lib = L
    return L


def check(rc: int, what: str) -> None:
    if rc != BK_OK:
        raise BKError(rc, what)


# ---- helpers -------------------------------------------------------------------

def _host(a) -> tuple:
    """A C double* to a contiguous float64 copy of `a` (kept alive by the
    returned tuple)."""
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    return arr, arr.ctypes.data_as(_dp)


def _ptr(t) -> int | None:
    if t is None:
        return None
    return t.data_ptr()


def _order(p: int, what: str) -> None:
    """bk::with_order (include/bk_common.h:162-178): orders 1..8."""
    if not 1 <= int(p) <= 8:
        raise BKError(BK_ERR_ORDER, f"{what}: p = {p}")


def _stream(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def order_q(bk: int, p: int) -> int:
    """Points per direction: p + 2 for BK1/BK3 (openmp/BK1.cpp:41), p + 1 for
    BK5 (openmp/BK5.cpp:153)."""
    return p + 1 if bk == 5 else p + 2


@dataclass
class ApplyOptions:
    prec: int = PREC_FP64
    engine: int = ENGINE_AUTO
    layout: int = LAYOUT_INTERLEAVED
    nfactors: int = 6
    elems_per_block: int = 0
    kernel: int = KERNEL_AUTO
    gform: int = G_STORAGE
    jxw_layout: int = JXW_PQR

    def c(self) -> Options:
        return Options(self.prec, self.engine, self.layout, self.nfactors, self.elems_per_block, self.kernel,
                       self.gform, self.jxw_layout)


# ---- operator apply (device tensors) -------------------------------------------

def bk1_apply(p, E, B, qdata, u, v, prec=PREC_FP64, engine=ENGINE_AUTO, jxw_layout=JXW_PQR, stream=None):
    """v = B^T diag(qdata) B u per element (openmp/bk1_sumfact.h:16-159);
    jxw_layout=JXW_RQP: qdata is JxW_t(e, r, q, p), as bk1_transpose_jxw
    (transpose_jxw, include/bk_harness.h:89-102) makes it."""
    _order(p, "bk1_apply")
    Bh, Bp = _host(B)
    o = ApplyOptions(prec=prec, engine=engine, jxw_layout=jxw_layout).c()
    check(lib().bk1_apply_opt(p, E, Bp, _ptr(qdata), _ptr(u), _ptr(v), C.byref(o), _stream(stream)), "bk1_apply")


def bk3_apply(p, E, B, D, G, u, v, k=None, prec=PREC_FP64, engine=ENGINE_AUTO, gform=G_STORAGE, stream=None):
    """v = B^T D^T (k) G D B u per element (openmp/bk3_sumfact.h:17-187); G
    factor-major, k an optional coefficient at the quadrature points.
    gform=G_FF: G holds the float-float pairs made by g_to_ff."""
    _order(p, "bk3_apply")
    Bh, Bp = _host(B)
    Dh, Dp = _host(D)
    o = ApplyOptions(prec=prec, engine=engine, gform=gform).c()
    check(lib().bk3_apply_k(p, E, Bp, Dp, _ptr(G), _ptr(k), _ptr(u), _ptr(v), C.byref(o), _stream(stream)),
          "bk3_apply")


def bk5_apply(p, E, D, G, u, v, prec=PREC_FP64, engine=ENGINE_AUTO, layout=LAYOUT_INTERLEAVED, nfactors=6,
              mass=None, lam=0.0, kernel=KERNEL_AUTO, elems_per_block=0, gform=G_STORAGE, stream=None):
    """v = D^T G D u (+ lam * mass * u) per element (openmp/BK5.cpp:18-103).
    gform=G_FF: G holds the float-float pairs made by g_to_ff."""
    _order(p, "bk5_apply")
    Dh, Dp = _host(D)
    o = ApplyOptions(prec=prec, engine=engine, layout=layout, nfactors=nfactors, kernel=kernel,
                     elems_per_block=elems_per_block, gform=gform).c()
    check(lib().bk5_apply_ex(p, E, Dp, _ptr(G), _ptr(u), _ptr(mass), float(lam), _ptr(v), C.byref(o),
                             _stream(stream)), "bk5_apply")


def bk5_make_g(p, E, G6i, nfactors=6, layout=LAYOUT_COLUMN, out=None, stream=None):
    """make_bk5_G (include/bk_harness.h:220-244) on the device: G6i in
    BK5.cpp's interleaved layout G6i(e, i, j, s, k) -> G with nfactors (6 or
    9) in `layout`; float64 tensors for FP64, float32 for the FP32 forms."""
    import torch
    q = p + 1
    if out is None:
        out = torch.empty(E * nfactors * q ** 3, dtype=G6i.dtype, device=G6i.device)
    prec = PREC_FP64 if G6i.dtype == torch.float64 else PREC_FP32
    check(lib().bk5_make_g(p, E, _ptr(G6i), _ptr(out), nfactors, layout, prec, _stream(stream)), "bk5_make_g")
    return out


def bk1_transpose_jxw(p, E, jxw, out=None, stream=None):
    """transpose_jxw (include/bk_harness.h:89-102) on the device: JxW(e, p,
    q, r) -> JxW_t(e, r, q, p), Q = p + 2; float64 or float32 tensors."""
    import torch
    if out is None:
        out = torch.empty_like(jxw)
    prec = PREC_FP64 if jxw.dtype == torch.float64 else PREC_FP32
    check(lib().bk1_transpose_jxw(p, E, _ptr(jxw), _ptr(out), prec, _stream(stream)), "bk1_transpose_jxw")
    return out


PROBE_COPY, PROBE_FF, PROBE_MMA = 0, 1, 2


def probe_contract(method, D, x, y, stream=None):
    """y(l, i) = sum_n D(i, n) x(l, n) over lines of 8 doubles by one route
    (include/bk_probe.h): PROBE_COPY (split and join only), PROBE_FF (the
    float-float route of the operator kernels) or PROBE_MMA (exact byte
    slices on the tensor cores); a measurement entry point."""
    Dh, Dp = _host(D)
    check(lib().bk_probe_contract(int(method), x.numel() // 8, Dp, _ptr(x), _ptr(y), _stream(stream)),
          "bk_probe_contract")
    return y


def bk5_set_auto_kernel(p, prec, layout, kernel, engine=ENGINE_AUTO, with_mass=False):
    """Fix the shape BK5's KERNEL_AUTO takes for (p, prec, engine, layout,
    mass term): KERNEL_SWEEP, KERNEL_COLUMN, or KERNEL_AUTO for the built-in
    rule (the tuner's hook, process-wide)."""
    check(lib().bk5_set_auto_kernel(p, prec, engine, layout, int(bool(with_mass)), kernel), "bk5_set_auto_kernel")


def bk5_auto_kernel(p, prec, layout, engine=ENGINE_AUTO, with_mass=False) -> int:
    """The shape BK5's KERNEL_AUTO takes for these arguments."""
    r = lib().bk5_auto_kernel(p, prec, engine, layout, int(bool(with_mass)))
    if r < 0:
        raise BKError(-r, "bk5_auto_kernel")
    return r


def g_to_ff(G, out=None, stream=None):
    """The float-float pairs of a float64 device tensor G (bk_g_to_ff): a
    tensor of G's shape and dtype float64 whose 8-byte values hold (float hi,
    float lo); in place when out is G.  For bk5_apply(..., gform=G_FF)."""
    if out is None:
        out = G.new_empty(G.shape)
    check(lib().bk_g_to_ff(_ptr(G), _ptr(out), G.numel(), _stream(stream)), "bk_g_to_ff")
    return out


def sum_factorization(bk: int, p: int, nelmt: int, *args, prec=PREC_FP64, **kw):
    """The reference's kernel interface: SumFactorization(nelmt, basis, JxW, in,
    out) for BK1, (nelmt, basis, dbasis, G, in, out) for BK3 and (nelmt,
    dbasis, G, in, out) for BK5, with the order p as a run-time argument."""
    if bk == 1:
        basis, jxw, inp, out = args
        return bk1_apply(p, nelmt, basis, jxw, inp, out, prec=prec, **kw)
    if bk == 3:
        basis, dbasis, G, inp, out = args
        return bk3_apply(p, nelmt, basis, dbasis, G, inp, out, prec=prec, **kw)
    if bk == 5:
        dbasis, G, inp, out = args
        return bk5_apply(p, nelmt, dbasis, G, inp, out, prec=prec, **kw)
    raise ValueError(f"unknown operator BK{bk}")


def device_status(reset: bool = True, stream=None) -> int:
    s = C.c_int(0)
    check(lib().bk_device_status(C.byref(s), 1 if reset else 0, _stream(stream)), "bk_device_status")
    return s.value


def version() -> str:
    return lib().bk_version().decode()


# ---- 1-D rules and matrices (host) ---------------------------------------------

def gauss(n: int):
    x = np.empty(n)
    w = np.empty(n)
    check(lib().bk_gauss_points(n, x.ctypes.data_as(_dp), w.ctypes.data_as(_dp)), "bk_gauss_points")
    return x, w


def gll(n: int):
    x = np.empty(n)
    w = np.empty(n)
    check(lib().bk_gll_points(n, x.ctypes.data_as(_dp), w.ctypes.data_as(_dp)), "bk_gll_points")
    return x, w


def lagrange_interp(nodes, pts):
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    B = np.empty(nodes.size * pts.size)
    check(lib().bk_lagrange_interp(nodes.size, nodes.ctypes.data_as(_dp), pts.size, pts.ctypes.data_as(_dp),
                                   B.ctypes.data_as(_dp)), "bk_lagrange_interp")
    return B


def lagrange_deriv(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    D = np.empty(x.size * x.size)
    check(lib().bk_lagrange_deriv(x.size, x.ctypes.data_as(_dp), D.ctypes.data_as(_dp)), "bk_lagrange_deriv")
    return D


def bk1_bk3_matrices(p: int):
    """(B, D_bk3, gauss x, gauss w, gll x) for BK1/BK3 at order p: P = p + 1
    GLL nodes, Q = p + 2 Gauss points; B(i, q) = l_i(x_q) (P x Q) and the BK3
    derivative D(n, q) = l_n'(x_q) on the Gauss points."""
    P, Q = p + 1, p + 2
    xn, _ = gll(P)
    xq, wq = gauss(Q)
    B = lagrange_interp(xn, xq)
    D = lagrange_deriv(xq).reshape(Q, Q).T.copy().ravel()
    return B, D, xq, wq, xn


def bk5_matrices(p: int):
    """(D, gll x, gll w) for BK5 at order p: Q = p + 1 GLL points, D(i, n) =
    l_n'(x_i)."""
    Q = p + 1
    x, w = gll(Q)
    return lagrange_deriv(x), x, w


# ---- seeded device inputs ------------------------------------------------------

def fill_uniform(t, seed: int, lo: float = -1.0, hi: float = 1.0, stream=None):
    import torch
    check(lib().bk_fill_uniform(_ptr(t), t.numel(), seed, lo, hi, int(t.dtype == torch.float64), _stream(stream)),
          "bk_fill_uniform")
    return t


def fill_lognormal(t, seed: int, sigma: float, stream=None):
    import torch
    check(lib().bk_fill_lognormal(_ptr(t), t.numel(), seed, sigma, int(t.dtype == torch.float64), _stream(stream)),
          "bk_fill_lognormal")
    return t


def geom_affine(Q, E, x, w, seed, h, pert, qdata=None, G=None, layout=LAYOUT_FACTOR, stream=None):
    xh, xp = _host(x)
    wh, wp = _host(w)
    check(lib().bk_geom_affine(Q, E, xp, wp, seed, h, pert, _ptr(qdata), _ptr(G), layout, _stream(stream)),
          "bk_geom_affine")


def coords_affine(Q, E, nx, ny, x, seed, h, pert, coords, stream=None):
    xh, xp = _host(x)
    check(lib().bk_coords_affine(Q, E, nx, ny, xp, seed, h, pert, _ptr(coords), _stream(stream)), "bk_coords_affine")


def geom_trilinear(Q, E, nx, ny, x, w, seed, h, jit, G=None, layout=LAYOUT_INTERLEAVED, mass=None, coords=None,
                   stream=None):
    xh, xp = _host(x)
    wh, wp = _host(w)
    check(lib().bk_geom_trilinear(Q, E, nx, ny, xp, wp, seed, h, jit, _ptr(G), layout, _ptr(mass), _ptr(coords),
                                  _stream(stream)), "bk_geom_trilinear")


def convert(src, dst, stream=None):
    import torch
    assert src.numel() == dst.numel()
    check(lib().bk_convert(_ptr(src), _ptr(dst), src.numel(), int(dst.dtype == torch.float32), _stream(stream)),
          "bk_convert")
    return dst


# ---- adjoint, vector kernels ---------------------------------------------------

def bk3_adjoint(p, E, B, D, G, k, u, res, dk, dG, prec=PREC_FP64, engine=ENGINE_AUTO, gform=G_STORAGE,
                stream=None):
    """dL/dk (E x Q^3) and dL/dG (E x 6 x Q^3) of L = 1/2 |A(k) u - f|^2 given
    res = A(k) u - f; the forward kernel is bk3_apply(..., k=k).  gform=G_FF:
    G holds the float-float pairs made by g_to_ff."""
    _order(p, "bk3_adjoint")
    Bh, Bp = _host(B)
    Dh, Dp = _host(D)
    o = ApplyOptions(prec=prec, engine=engine, gform=gform).c()
    check(lib().bk3_adjoint(p, E, Bp, Dp, _ptr(G), _ptr(k), _ptr(u), _ptr(res), _ptr(dk), _ptr(dG), C.byref(o),
                            _stream(stream)), "bk3_adjoint")


STREAM_COPY, STREAM_TRIAD, STREAM_MIX = 0, 1, 2


def stream_kernel(kind, a, b, c=None, reads=1, stream=None):
    nbytes = a.numel() * a.element_size()
    check(lib().bk_stream_kernel(kind, nbytes, _ptr(a), _ptr(b), _ptr(c), reads, _stream(stream)),
          "bk_stream_kernel")


def dot_workspace(n, device="cuda"):
    import torch
    return torch.empty(int(lib().bk_dot_workspace_bytes(n)) // 8, dtype=torch.float64, device=device)


def dot(x, y, out, workspace, half=False, stream=None):
    """out[0] = x . y (FP64 accumulation, deterministic); out a device double."""
    import torch
    check(lib().bk_dot(x.numel(), _ptr(x), _ptr(y), int(x.dtype == torch.float64), _ptr(out), _ptr(workspace),
                       workspace.numel() * 8, int(half), _stream(stream)), "bk_dot")
    return out


def axpby(a, x, b, y, stream=None):
    """y = a x + b y."""
    import torch
    check(lib().bk_axpby(x.numel(), float(a), _ptr(x), float(b), _ptr(y), int(y.dtype == torch.float64),
                         _stream(stream)), "bk_axpby")
    return y


# ---- applies on host arrays (include/bk_host.h) ------------------------------------

class HostPlan:
    """Applies of operator `op` (1, 3, 5) at order p over E elements whose u
    and v live in HOST memory (pinned for overlap): element chunks go
    host -> device -> apply -> host on three streams.  G/qdata/k stay on the
    device.  apply() is asynchronous on `stream`; synchronize it before
    reading v."""

    def __init__(self, op, p, E, prec=PREC_FP64, chunk_elems=0):
        L = lib()
        if not getattr(L, "_host_declared", False):
            L.bk_host_plan_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int64, C.c_int, C.c_int64]
            L.bk_host_plan_destroy.argtypes = [C.c_void_p]
            L.bk1_apply_host.argtypes = [C.c_void_p, _dp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p]
            L.bk3_apply_host.argtypes = [C.c_void_p, _dp, _dp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p]
            L.bk5_apply_host.argtypes = [C.c_void_p, _dp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p]
            L._host_declared = True
        self.op, self.p, self.E, self.prec = int(op), int(p), int(E), prec
        h = C.c_void_p()
        check(L.bk_host_plan_create(C.byref(h), self.op, self.p, self.E, prec, int(chunk_elems)),
              "bk_host_plan_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().bk_host_plan_destroy(self.h)
            self.h = None

    __del__ = close

    def apply(self, u_host, v_host, G=None, B=None, D=None, k=None, engine=ENGINE_AUTO,
              layout=LAYOUT_INTERLEAVED, nfactors=6, kernel=KERNEL_AUTO, jxw_layout=JXW_PQR, stream=None):
        """v_host = A u_host (torch CPU tensors or numpy arrays); G: qdata
        (BK1) or the geometric factors (BK3, BK5) on the device."""
        o = ApplyOptions(prec=self.prec, engine=engine, layout=layout, nfactors=nfactors, kernel=kernel,
                         jxw_layout=jxw_layout).c()
        uptr = u_host.data_ptr() if hasattr(u_host, "data_ptr") else u_host.ctypes.data
        vptr = v_host.data_ptr() if hasattr(v_host, "data_ptr") else v_host.ctypes.data
        L = lib()
        if self.op == 1:
            Bh, Bp = _host(B)
            rc = L.bk1_apply_host(self.h, Bp, _ptr(G), uptr, vptr, C.byref(o), _stream(stream))
        elif self.op == 3:
            Bh, Bp = _host(B)
            Dh, Dp = _host(D)
            rc = L.bk3_apply_host(self.h, Bp, Dp, _ptr(G), _ptr(k), uptr, vptr, C.byref(o), _stream(stream))
        else:
            Dh, Dp = _host(D)
            rc = L.bk5_apply_host(self.h, Dp, _ptr(G), uptr, vptr, C.byref(o), _stream(stream))
        check(rc, f"bk{self.op}_apply_host")
