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


# ---- inputs of the benchmark configurations (oracle/bk_geom_oracle.c) --------

def test_splitmix64_known_values(oracle_lib):
    """splitmix64 (Steele, Lea, Flood 2014) from state 0: the generator's
    published first outputs."""
    L = oracle_lib.lib()
    assert L.bko_splitmix64(0) == 0xE220A8397B1DCDAF
    assert L.bko_splitmix64(0x9E3779B97F4A7C15) == 0x6E789E6AA1B965F4
    # U(s, i): the top 53 bits over 2^53
    s = L.bko_splitmix64(5)
    assert L.bko_uniform01(5, 3) == (L.bko_splitmix64((s + 3) % 2 ** 64) >> 11) / 2.0 ** 53
    u = oracle_lib.uniform(100000, 9)
    assert -1.0 <= u.min() and u.max() < 1.0 and abs(u.mean()) < 0.01


@pytest.mark.parametrize("n", range(2, 11))
def test_rules(oracle_lib, n):
    o = oracle_lib
    xg, wg = o.gauss(n)
    xr, wr = np.polynomial.legendre.leggauss(n)
    assert np.abs(xg - xr).max() < 1e-14 and np.abs(wg - wr).max() < 1e-14
    x, w = o.gll(n)
    inner = np.sort(np.polynomial.legendre.Legendre.basis(n - 1).deriv().roots().real)
    assert x[0] == -1.0 and x[-1] == 1.0 and (n == 2 or np.abs(x[1:-1] - inner).max() < 1e-13)
    # GLL is exact for degree 2n - 3
    for k in range(2 * n - 2):
        exact = 0.0 if k % 2 else 2.0 / (k + 1)
        assert abs(w @ x ** k - exact) < 1e-14
    D = o.lagrange_deriv(x).reshape(n, n)
    assert np.abs(D @ np.ones(n)).max() < 1e-12 and np.abs(D @ x - 1).max() < 1e-12
    B = o.lagrange_interp(x, xg).reshape(n, n)   # B(i, q) = l_i(xg_q)
    assert np.abs(B.sum(axis=0) - 1).max() < 1e-14 and np.abs(x @ B - xg).max() < 1e-14


def test_affine_geometry_analytic(oracle_lib):
    """Undistorted affine elements (pert = 0): J = (h/2) I, so qdata = w h^3/8
    (summing to h^3 per element) and G = w (h/2) I."""
    o = oracle_lib
    Q, h, E = 5, 1.0 / 16, 3
    x, w = o.gauss(Q)
    q, G = o.geom_affine(Q, 0, E, x, w, 21, h, 0.0)
    W = np.einsum("i,j,k->ijk", w, w, w).ravel()
    assert np.abs(q.reshape(E, -1).sum(axis=1) - h ** 3).max() < 1e-15
    G = G.reshape(E, 6, -1)
    for f, diag in enumerate((1, 0, 0, 1, 0, 1)):
        assert np.abs(G[:, f] - diag * W * h / 2).max() <= 1e-16


def test_affine_geometry_against_numpy(oracle_lib):
    """G = w det J J^-1 J^-T with J from the stated seeded perturbation,
    formed here by numpy's inverse (a third formula)."""
    o = oracle_lib
    Q, h, pert, seed, E = 4, 1.0 / 16, 0.2, 41, 5
    x, w = o.gauss(Q)
    q, G = o.geom_affine(Q, 0, E, x, w, seed, h, pert, layout=1)
    L = o.lib()
    G = G.reshape(E, Q, Q, 6, Q)
    for e in range(E):
        P = np.array([[2 * L.bko_uniform01(seed, 9 * e + 3 * a + b) - 1 for b in range(3)] for a in range(3)])
        J = 0.5 * h * (np.eye(3) + pert * P)
        K = np.linalg.inv(J)
        M = np.linalg.det(J) * K @ K.T
        for i, j, k in ((0, 0, 0), (1, 2, 3), (3, 3, 1)):
            wp = w[i] * w[j] * w[k]
            ref = wp * np.array([M[0, 0], M[0, 1], M[0, 2], M[1, 1], M[1, 2], M[2, 2]])
            assert np.abs(G[e, i, j, :, k] - ref).max() <= 1e-14 * np.abs(ref).max()
            assert abs(q[(e * Q + i) * Q * Q + j * Q + k] - wp * np.linalg.det(J)) <= 1e-14 * wp * h ** 3


def test_trilinear_geometry(oracle_lib):
    """Without jitter the trilinear map of a grid cell is the affine map
    x = c + (h/2) xi: G = w (h/2) I and the coordinates follow; with jitter
    the three layouts hold the same factors and the mass is w det J."""
    o = oracle_lib
    Q, h, nx = 4, 0.25, 3
    x, w = o.gll(Q)
    G, m, c = o.geom_trilinear(Q, 0, 30, nx, nx, x, w, 5, h, 0.0, layout=0, mass=True, coords=True)
    W = np.einsum("i,j,k->ijk", w, w, w).ravel()
    G = G.reshape(30, 6, -1)
    for f, diag in enumerate((1, 0, 0, 1, 0, 1)):
        assert np.abs(G[:, f] - diag * W * h / 2).max() <= 1e-15
    assert np.abs(m.reshape(30, -1) - W * h ** 3 / 8).max() <= 1e-16
    c = c.reshape(30, Q, Q, Q, 3)
    e = 23   # cell (2, 1, 2)
    assert abs(c[e, 1, 2, 3, 0] - (2.5 + 0.5 * x[1]) * h) < 1e-15
    assert abs(c[e, 1, 2, 3, 1] - (1.5 + 0.5 * x[2]) * h) < 1e-15
    assert abs(c[e, 1, 2, 3, 2] - (2.5 + 0.5 * x[3]) * h) < 1e-15
    # jittered: the three layouts are permutations of one another
    g = [o.geom_trilinear(Q, 7, 4, nx, nx, x, w, 5, h, 0.15, layout=L)[0].reshape(4, -1) for L in (0, 1, 2)]
    g0 = g[0].reshape(4, 6, Q, Q, Q)
    assert np.array_equal(np.ascontiguousarray(g0.transpose(0, 2, 3, 1, 4)).reshape(4, -1), g[1])
    assert np.array_equal(np.ascontiguousarray(g0.transpose(0, 1, 4, 2, 3)).reshape(4, -1), g[2])
    # an element range gives the same elements as the full array
    full = o.geom_trilinear(Q, 0, 11, nx, nx, x, w, 5, h, 0.15, layout=1)[0].reshape(11, -1)
    assert np.array_equal(full[7:11], g[1])
