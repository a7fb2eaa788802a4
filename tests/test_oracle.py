"""The oracle (oracle/bk_oracle.c) pinned to the reference's own kernels:
tests/golden holds outputs of the reference's SumFactorization<double, nq>,
its harness references and layout helpers, compiled from its sources
(tests/golden/make_golden.py)."""
import numpy as np
import pytest

P_ALL = list(range(1, 9))


def _sizes(bk, p):
    nq = p + 1 if bk == 5 else p + 2
    nm = nq if bk == 5 else nq - 1
    ngeo = nq ** 3 if bk == 1 else 6 * nq ** 3
    return nq, nm, ngeo


def test_lcg_and_test_basis(oracle_lib, golden):
    arr, meta = golden
    o = oracle_lib
    a, _ = o.random_test_data(32, 0, meta["seed"])
    assert np.array_equal(a, arr["lcg_first_32"])
    assert np.array_equal(o.test_basis(4, 5), arr["test_basis_4x5_f64"])
    assert np.array_equal(o.test_basis(4, 5, np.float32).astype(np.float64), arr["test_basis_4x5_f32"])


@pytest.mark.parametrize("bk", [1, 3, 5])
@pytest.mark.parametrize("p", P_ALL)
def test_sumfact_random_f64(oracle_lib, golden, bk, p):
    """bk_oracle.c's restatement of SumFactorization<double> against the
    reference's own kernel on the reference's random test data."""
    arr, meta = golden
    o = oracle_lib
    E = meta["E_rand"]
    nq, nm, ngeo = _sizes(bk, p)
    u, g = o.random_test_data(E * nm ** 3, E * ngeo, meta["seed"])
    if bk == 1:
        out = o.bk1(nq, E, o.test_basis(nm, nq), g, u)
    elif bk == 3:
        out = o.bk3(nq, E, o.test_basis(nm, nq), o.test_basis(nq, nq), g, u)
    else:
        out = o.bk5(nq, E, o.test_basis(nq, nq), g, u)
    ref = arr[f"bk{bk}_p{p}_rand_f64"]
    assert o.rel_maxdiff(out, ref) < 1e-14


@pytest.mark.parametrize("bk", [1, 3, 5])
@pytest.mark.parametrize("p", P_ALL)
def test_harness_reference(oracle_lib, golden, bk, p):
    """reference_bk1/3/5 (float inputs, double arithmetic)."""
    arr, meta = golden
    o = oracle_lib
    E = meta["E_rand"]
    nq, nm, ngeo = _sizes(bk, p)
    u, g = o.random_test_data(E * nm ** 3, E * ngeo, meta["seed"])
    uf, gf = u.astype(np.float32), g.astype(np.float32)
    if bk == 1:
        out = o.reference_bk1(nq, E, o.test_basis(nm, nq, np.float32), gf, uf)
    elif bk == 3:
        out = o.reference_bk3(nq, E, o.test_basis(nm, nq, np.float32), o.test_basis(nq, nq, np.float32), gf, uf)
    else:
        out = o.reference_bk5(nq, E, o.test_basis(nq, nq, np.float32), gf, uf)
    assert o.rel_maxdiff(out, arr[f"bk{bk}_p{p}_harness"]) < 1e-14


@pytest.mark.parametrize("bk", [1, 3, 5])
@pytest.mark.parametrize("p", P_ALL)
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_constant_data_norm(oracle_lib, golden, bk, p, prec):
    """The drivers' known answer: in = 3, JxW = 1 / G = 2, cos test basis, the
    printed "norm =" (openmp/BK1.cpp:40-44, BK3.cpp:56-60, BK5.cpp:118-120)."""
    arr, meta = golden
    o = oracle_lib
    E = meta["E_const"]
    nq, nm, ngeo = _sizes(bk, p)
    dt = np.float32 if prec == "f32" else np.float64
    u = np.full(E * nm ** 3, 3.0, dtype=dt)
    g = np.full(E * ngeo, 1.0 if bk == 1 else 2.0, dtype=dt)
    if bk == 1:
        out = o.bk1(nq, E, o.test_basis(nm, nq, dt), g, u)
    elif bk == 3:
        out = o.bk3(nq, E, o.test_basis(nm, nq, dt), o.test_basis(nq, nq, dt), g, u)
    else:
        out = o.bk5(nq, E, o.test_basis(nq, nq, dt), g, u)
    ref = meta["norms"][f"bk{bk}_p{p}_const_{prec}"]
    tol = 2e-5 if prec == "f32" else 1e-13
    assert abs(o.norm2(out) - ref) <= tol * abs(ref)


@pytest.mark.parametrize("F", [6, 9])
@pytest.mark.parametrize("layout", [0, 1, 2])
def test_make_bk5_G(oracle_lib, golden, F, layout):
    arr, _ = golden
    o = oracle_lib
    nq = 3
    g6i = o.random_test_data(0, 6 * nq ** 3)[1].astype(np.float32).astype(np.float64)
    G = o.make_bk5_G(g6i, 1, nq, F, layout)
    assert np.array_equal(G, arr[f"make_bk5_G_nq3_F{F}_L{layout}"])


def test_transpose_jxw(oracle_lib, golden):
    arr, _ = golden
    o = oracle_lib
    jx = o.random_test_data(0, 4 ** 3)[1].astype(np.float32).astype(np.float64)
    assert np.array_equal(o.transpose_jxw(jx, 1, 4), arr["transpose_jxw_nq4"])


def test_bk5_layouts_agree(oracle_lib):
    """BK5 with G built in every layout equals BK5 on the interleaved G after
    the matching relayout (the G6/G9 equivalence of bk5_offload.cpp:26-27)."""
    o = oracle_lib
    nq, E = 4, 3
    u, g6i = o.random_test_data(E * nq ** 3, E * 6 * nq ** 3, 7)
    D = o.test_basis(nq, nq)
    ref = o.bk5(nq, E, D, g6i, u)
    # back from layout 0 (factor-major) to interleaved by the inverse permutation
    G0 = o.make_bk5_G(g6i, E, nq, 6, 0).reshape(E, 6, nq, nq, nq)
    back = np.ascontiguousarray(G0.transpose(0, 2, 3, 1, 4)).ravel()
    assert np.array_equal(back, g6i)
    assert o.rel_maxdiff(o.bk5(nq, E, D, back, u), ref) == 0.0


def test_adjoint_oracle_fd(oracle_lib):
    """The FP64 host gradient of L = 1/2 |A(k) u - f|^2 (no reference
    counterpart) against central finite differences in k and in G."""
    o = oracle_lib
    rng = np.random.default_rng(3)
    p, E = 2, 2
    nq, nm = p + 2, p + 1
    B = o.test_basis(nm, nq) * 0.3
    D = o.test_basis(nq, nq) * 0.3
    G = rng.uniform(0.5, 1.5, E * 6 * nq ** 3)
    k = np.exp(rng.normal(0, 0.5, E * nq ** 3))
    u = rng.uniform(-1, 1, E * nm ** 3)
    f = rng.uniform(-1, 1, E * nm ** 3)

    def loss(k_, G_):
        r = o.bk3(nq, E, B, D, G_, u, k=k_) - f
        return 0.5 * float(r @ r)

    res = o.bk3(nq, E, B, D, G, u, k=k) - f
    dk, dG = o.bk3_adjoint(nq, E, B, D, G, k, u, res)
    h = 1e-6
    for _ in range(8):
        d = rng.standard_normal(k.size)
        fd = (loss(k + h * d, G) - loss(k - h * d, G)) / (2 * h)
        assert abs(fd - dk @ d) <= 1e-7 * max(1.0, abs(fd))
        dg = rng.standard_normal(G.size)
        fd = (loss(k, G + h * dg) - loss(k, G - h * dg)) / (2 * h)
        assert abs(fd - dG @ dg) <= 1e-7 * max(1.0, abs(fd))
