"""Size-independent properties of the operators at the configurations' full
sizes, where the oracle is too slow to compare entry by entry:

  - BK5 p=7, E = 262144 (134 M points, the headline): A 1 = 0 (constants are
    in the Laplacian's kernel), symmetry u.Aw = w.Au, linearity
    A(u + 2w) = Au + 2Aw, FP64 forms against each other (float-float vs
    native DFMA) and the mixed form's error;
  - BK3 p=6, E = 131072: A 1 = 0 and symmetry;
  - BK1 p=3, E = 4096: 1.M1 = sum of qdata (B's columns sum to one) and
    symmetry.
Thresholds are relative to |A| |u| style scales (stated per test)."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _dot(a, b):
    return float(torch.dot(a.double(), b.double()))


@pytest.fixture(scope="module")
def bk5_full(bklib):
    bk = bklib
    p, E, nx = 7, 262144, 64
    Q = p + 1
    D, x, w = bk.bk5_matrices(p)
    G = torch.empty(E * 6 * Q ** 3, dtype=torch.float64, device="cuda")
    bk.geom_trilinear(Q, E, nx, nx, x, w, 2, 1.0 / nx, 0.15, G=G, layout=bk.LAYOUT_COLUMN)
    u = bk.fill_uniform(torch.empty(E * Q ** 3, dtype=torch.float64, device="cuda"), 11)
    wv = bk.fill_uniform(torch.empty_like(u), 12)
    yield p, E, D, G, u, wv
    del G


def _bk5(bk, p, E, D, G, x, **kw):
    y = torch.empty_like(x)
    bk.bk5_apply(p, E, D, G, x, y, layout=bk.LAYOUT_COLUMN, **kw)
    return y


def test_bk5_full_constants_in_kernel(bklib, bk5_full):
    p, E, D, G, u, _ = bk5_full
    Au = _bk5(bklib, p, E, D, G, u)
    A1 = _bk5(bklib, p, E, D, G, torch.ones_like(u))
    # |A 1| against the size of A u for u ~ U[-1, 1]
    assert float(A1.abs().max()) <= 1e-12 * float(Au.abs().max())


def test_bk5_full_symmetry_linearity(bklib, bk5_full):
    bk = bklib
    p, E, D, G, u, w = bk5_full
    Au, Aw = _bk5(bk, p, E, D, G, u), _bk5(bk, p, E, D, G, w)
    uAw, wAu = _dot(u, Aw), _dot(w, Au)
    scale = float(torch.linalg.norm(u) * torch.linalg.norm(Aw))
    assert abs(uAw - wAu) <= 1e-12 * scale
    A_lin = _bk5(bk, p, E, D, G, u + 2 * w)
    assert float((A_lin - Au - 2 * Aw).abs().max()) <= 1e-12 * float(A_lin.abs().max())


def test_bk5_full_forms_agree(bklib, bk5_full):
    bk = bklib
    p, E, D, G, u, _ = bk5_full
    ff = _bk5(bk, p, E, D, G, u, engine=bk.ENGINE_FF)
    dfma = _bk5(bk, p, E, D, G, u, engine=bk.ENGINE_DFMA)
    big = float(dfma.abs().max())
    assert float((ff - dfma).abs().max()) <= 1e-12 * big
    u32, G32 = u.float(), G.float()
    for prec in (bk.PREC_MIXED, bk.PREC_FP32):
        v32 = torch.empty_like(u32)
        bk.bk5_apply(p, E, D, G32, u32, v32, prec=prec, layout=bk.LAYOUT_COLUMN)
        assert float((v32.double() - dfma).abs().max()) <= 1e-5 * big


def test_bk3_full_constants_and_symmetry(bklib):
    bk = bklib
    p, E = 6, 131072
    P, Q = p + 1, p + 2
    B, Dm, xq, wq, _ = bk.bk1_bk3_matrices(p)
    G = torch.empty(E * 6 * Q ** 3, dtype=torch.float64, device="cuda")
    bk.geom_affine(Q, E, xq, wq, 31, 1.0 / 64, 0.2, G=G, layout=bk.LAYOUT_FACTOR)
    u = bk.fill_uniform(torch.empty(E * P ** 3, dtype=torch.float64, device="cuda"), 32)
    w = bk.fill_uniform(torch.empty_like(u), 33)
    ap = lambda x: (lambda y: (bk.bk3_apply(p, E, B, Dm, G, x, y), y)[1])(torch.empty_like(x))
    Au, Aw, A1 = ap(u), ap(w), ap(torch.ones_like(u))
    assert float(A1.abs().max()) <= 1e-12 * float(Au.abs().max())
    scale = float(torch.linalg.norm(u) * torch.linalg.norm(Aw))
    assert abs(_dot(u, Aw) - _dot(w, Au)) <= 1e-12 * scale


def test_bk1_full_mass_and_symmetry(bklib):
    bk = bklib
    p, E = 3, 4096
    P, Q = p + 1, p + 2
    B, _, xq, wq, _ = bk.bk1_bk3_matrices(p)
    qd = torch.empty(E * Q ** 3, dtype=torch.float64, device="cuda")
    bk.geom_affine(Q, E, xq, wq, 21, 1.0 / 16, 0.2, qdata=qd)
    one = torch.ones(E * P ** 3, dtype=torch.float64, device="cuda")
    M1 = torch.empty_like(one)
    bk.bk1_apply(p, E, B, qd, one, M1)
    # 1.M1 = sum over the points of qdata: the interpolation reproduces 1
    assert abs(float(M1.sum()) - float(qd.sum())) <= 1e-12 * float(qd.sum())
    u = bk.fill_uniform(torch.empty_like(one), 22)
    w = bk.fill_uniform(torch.empty_like(one), 23)
    Mu, Mw = torch.empty_like(u), torch.empty_like(w)
    bk.bk1_apply(p, E, B, qd, u, Mu)
    bk.bk1_apply(p, E, B, qd, w, Mw)
    scale = float(torch.linalg.norm(u) * torch.linalg.norm(Mw))
    assert abs(_dot(u, Mw) - _dot(w, Mu)) <= 1e-12 * scale
