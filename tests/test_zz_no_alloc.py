"""bk_dot_noalloc: the FP64 dot product for callers that cannot allocate
device memory (for example code that runs while a stream is captured into a
CUDA graph, or a host whose device memory belongs to another runtime's pool),
with its partial sums in a fixed array of the library instead of a
caller-provided workspace.

Checked through the C ABI against the existing entry point bk_dot (which
takes a workspace), within the dot-product tolerance of the other tests, on
two calls in a row -- a long vector, then a short one, so that partial sums
left in the shared array by the first call must not leak into the second --
and in both storage types.  Collected last so that a failure here stops a
-x run only after every other test has run; it also passes on its own in a
fresh process (the first call does the per-device set-up).
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _noalloc(bklib):
    L = bklib.lib()
    f = L.bk_dot_noalloc
    f.argtypes = [C.c_longlong, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]
    f.restype = C.c_int
    return f, 268_435_456   # BK_DOT_NOALLOC_MAX_N of include/bk_vec.h


def _ref_dot(bklib, x, y, half):
    ws = bklib.dot_workspace(x.numel())
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    bklib.dot(x, y, out, ws, half=half)
    return out


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_noalloc_dot_matches_workspace_dot(bklib, dtype):
    f, nmax = _noalloc(bklib)
    assert nmax == 4096 * 65536
    s = torch.cuda.current_stream().cuda_stream
    f64 = int(dtype == torch.float64)
    for n, seed, half in ((3_000_001, 11, 0), (1000, 12, 1)):
        x = bklib.fill_uniform(torch.empty(n, dtype=dtype, device="cuda"), seed)
        y = bklib.fill_uniform(torch.empty(n, dtype=dtype, device="cuda"), seed + 100)
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        assert f(n, x.data_ptr(), y.data_ptr(), f64, out.data_ptr(), half, s) == bklib.BK_OK
        ref = _ref_dot(bklib, x, y, bool(half))
        torch.cuda.synchronize()
        scale = float((x.double() * y.double()).abs().sum())
        assert abs(out.item() - ref.item()) <= 1e-12 * max(1.0, scale), (n, out.item(), ref.item())
        exact = float(np.dot(x.double().cpu().numpy(), y.double().cpu().numpy())) * (0.5 if half else 1.0)
        assert abs(out.item() - exact) <= 1e-12 * max(1.0, scale)


def test_noalloc_dot_limits(bklib):
    f, nmax = _noalloc(bklib)
    s = torch.cuda.current_stream().cuda_stream
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    # beyond the fixed scratch: rejected before any launch
    assert f(nmax + 1, x.data_ptr(), x.data_ptr(), 1, out.data_ptr(), 0, s) == bklib.BK_ERR_SIZE
    assert f(-1, x.data_ptr(), x.data_ptr(), 1, out.data_ptr(), 0, s) == bklib.BK_ERR_SIZE
    assert f(8, x.data_ptr(), x.data_ptr(), 1, None, 0, s) == bklib.BK_ERR_NULL
    # an empty dot is zero
    out.fill_(7.0)
    assert f(0, None, None, 1, out.data_ptr(), 0, s) == bklib.BK_OK
    torch.cuda.synchronize()
    assert out.item() == 0.0
