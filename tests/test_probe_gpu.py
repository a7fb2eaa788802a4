"""The contraction probe (include/bk_probe.h): the float-float route and the
tensor-core route by exact byte slices both give FP64-accurate D x for the
BK5 p = 7 GLL derivative, on U[-1,1] lines and on lines whose values span
many binades (the slices are aligned per line), against numpy's FP64 product.

Tolerance: |y - ref| <= 1e-13 (sum_n |D(i,n)|) max_n |x(n)| per output --
normwise per line, because the tensor-core route aligns a line's mantissas
to its largest exponent (the float-float route meets it too); the copy route
reproduces x to float-float accuracy (2^-47)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _lines(n, seed, spread):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, 8))
    if spread:
        x *= 2.0 ** rng.integers(-spread, spread + 1, (n, 8))
    return x


@pytest.mark.parametrize("spread", [0, 20])
@pytest.mark.parametrize("method", ["ff", "mma"])
def test_probe_contract(bklib, method, spread):
    D = bklib.bk5_matrices(7)[0].reshape(8, 8)
    x = _lines(4096, 5 + spread, spread)
    xd = torch.from_numpy(x.ravel()).cuda()
    y = torch.full_like(xd, float("nan"))
    m = bklib.PROBE_FF if method == "ff" else bklib.PROBE_MMA
    bklib.probe_contract(m, D, xd, y)
    torch.cuda.synchronize()
    got = y.cpu().numpy().reshape(-1, 8)
    ref = x @ D.T
    bound = np.abs(D).sum(axis=1)[None, :] * np.abs(x).max(axis=1)[:, None]
    assert np.all(np.abs(got - ref) <= 1e-13 * bound), float(np.max(np.abs(got - ref) / bound))


def test_probe_copy_and_arguments(bklib):
    import ctypes as C
    D = bklib.bk5_matrices(7)[0]
    x = _lines(1000, 3, 4)
    xd = torch.from_numpy(x.ravel()).cuda()
    y = torch.empty_like(xd)
    bklib.probe_contract(bklib.PROBE_COPY, D, xd, y)
    torch.cuda.synchronize()
    assert np.all(np.abs(y.cpu().numpy() - x.ravel()) <= 2.0 ** -47 * np.abs(x.ravel()))
    L = bklib.lib()
    Dh = np.ascontiguousarray(D)
    dp = Dh.ctypes.data_as(C.POINTER(C.c_double))
    assert L.bk_probe_contract(2, 1000, dp, xd.data_ptr(), y.data_ptr(), None) == bklib.BK_ERR_SIZE   # not x16
    assert L.bk_probe_contract(3, 16, dp, xd.data_ptr(), y.data_ptr(), None) == bklib.BK_ERR_ARG
    assert L.bk_probe_contract(1, 16, dp, None, y.data_ptr(), None) == bklib.BK_ERR_NULL
    # the float-float route needs a centro-antisymmetric D
    Dn = np.ascontiguousarray(np.arange(64, dtype=np.float64))
    assert L.bk_probe_contract(1, 16, Dn.ctypes.data_as(C.POINTER(C.c_double)), xd.data_ptr(), y.data_ptr(),
                               None) == bklib.BK_ERR_ARG
