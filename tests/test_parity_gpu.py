"""Parity of the CUDA kernels with the oracle (the reference's algorithm
restated in C, pinned to the reference's own kernels) and with the golden
vectors of the reference itself.

Tolerances (largest |out - ref| over the largest |ref|, the reference's
rel_maxdiff, include/bk_harness.h:74-83):
  FP64 engines (DFMA, float-float)     1e-12  (the target of the work)
  FP32 storage (FP32, MIXED)           1e-5   (the reference's fail_mark)
"""
import numpy as np
import pytest
import torch

import oracle
from gpu_util import dev, gpu_apply, host, oracle_apply, random_case, sizes

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5
P_ALL = list(range(1, 9))


@pytest.fixture(scope="module", autouse=True)
def _cuda(bklib):
    assert torch.cuda.is_available(), "the GPU tests need CUDA: the product has no CPU path"
    bklib.device_status(reset=True)
    yield
    assert bklib.device_status(reset=True) == bklib.BK_OK


@pytest.mark.parametrize("bk", [1, 3, 5])
@pytest.mark.parametrize("p", P_ALL)
@pytest.mark.parametrize("engine", ["dfma", "ff"])
def test_fp64_random(bklib, bk, p, engine):
    E = 13
    nq, basis, dbasis, g, u = random_case(bk, p, E)
    eng = bklib.ENGINE_DFMA if engine == "dfma" else bklib.ENGINE_FF
    out = gpu_apply(bklib, bk, p, E, basis, dbasis, g, u, bklib.PREC_FP64, engine=eng)
    ref = oracle_apply(bk, nq, E, basis, dbasis, g, u)
    assert np.all(np.isfinite(out))
    assert oracle.rel_maxdiff(out, ref) < TOL64


@pytest.mark.parametrize("bk", [1, 3, 5])
@pytest.mark.parametrize("p", P_ALL)
@pytest.mark.parametrize("prec", ["fp32", "mixed"])
def test_fp32_random(bklib, bk, p, prec):
    E = 13
    nq, basis, dbasis, g, u = random_case(bk, p, E)
    pr = bklib.PREC_FP32 if prec == "fp32" else bklib.PREC_MIXED
    out = gpu_apply(bklib, bk, p, E, basis, dbasis, g, u, pr)
    # the FP32 kernels read the inputs rounded to float
    ref = oracle_apply(bk, nq, E, basis, dbasis, g.astype(np.float32), u.astype(np.float32))
    assert np.all(np.isfinite(out))
    assert oracle.rel_maxdiff(out, ref) < TOL32


@pytest.mark.parametrize("bk", [1, 3, 5])
@pytest.mark.parametrize("p", P_ALL)
def test_golden_vectors(bklib, golden, bk, p):
    """Against the reference's own SumFactorization<double, nq> outputs."""
    arr, meta = golden
    E = meta["E_rand"]
    nq, basis, dbasis, g, u = random_case(bk, p, E, meta["seed"])
    out = gpu_apply(bklib, bk, p, E, basis, dbasis, g, u, bklib.PREC_FP64)
    assert oracle.rel_maxdiff(out, arr[f"bk{bk}_p{p}_rand_f64"]) < TOL64


@pytest.mark.parametrize("bk", [1, 3, 5])
@pytest.mark.parametrize("p", P_ALL)
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_constant_data_norm(bklib, golden, bk, p, prec):
    """The drivers' known answer: "norm =" on constant data (in = 3, JxW = 1,
    G = 2, cos basis) as printed by the reference's BK1/BK3/BK5."""
    arr, meta = golden
    E = meta["E_const"]
    nq, nm, ngeo = sizes(bk, p)
    dt = np.float32 if prec == "f32" else np.float64
    u = np.full(E * nm ** 3, 3.0)
    g = np.full(E * ngeo, 1.0 if bk == 1 else 2.0)
    basis = oracle.test_basis(nm, nq, dt).astype(np.float64) if bk != 5 else None
    dbasis = oracle.test_basis(nq, nq, dt).astype(np.float64) if bk != 1 else None
    pr = bklib.PREC_FP32 if prec == "f32" else bklib.PREC_FP64
    out = gpu_apply(bklib, bk, p, E, basis, dbasis, g, u, pr)
    ref = meta["norms"][f"bk{bk}_p{p}_const_{prec}"]
    nrm = float(np.sqrt(np.sum(out * out)))
    assert abs(nrm - ref) <= (2e-5 if prec == "f32" else 1e-12) * abs(ref)
    e0 = arr[f"bk{bk}_p{p}_const_{prec}_e0"]
    assert oracle.rel_maxdiff(out[: e0.size], e0) < (TOL32 if prec == "f32" else TOL64)


@pytest.mark.parametrize("E", [1, 2, 3, 5, 16, 33, 100])
@pytest.mark.parametrize("bk,p", [(1, 3), (3, 6), (5, 7), (5, 8), (3, 8)])
def test_element_counts(bklib, bk, p, E):
    """Any element count: partial last batches, batches whose slices start off
    a 16-byte boundary (the TMA head/tail path)."""
    nq, basis, dbasis, g, u = random_case(bk, p, E, seed=E)
    for prec, tol in ((bklib.PREC_FP64, TOL64), (bklib.PREC_FP32, TOL32)):
        out = gpu_apply(bklib, bk, p, E, basis, dbasis, g, u, prec)
        if prec == bklib.PREC_FP32:
            ref = oracle_apply(bk, nq, E, basis, dbasis, g.astype(np.float32), u.astype(np.float32))
        else:
            ref = oracle_apply(bk, nq, E, basis, dbasis, g, u)
        assert oracle.rel_maxdiff(out, ref) < tol


@pytest.mark.parametrize("p", [1, 4, 7, 8])
@pytest.mark.parametrize("nfactors", [6, 9])
@pytest.mark.parametrize("layout", [0, 1, 2])
@pytest.mark.parametrize("engine", ["dfma", "ff", "fp32"])
@pytest.mark.parametrize("kernel", ["sweep", "column"])
def test_bk5_layouts(bklib, p, nfactors, layout, engine, kernel):
    """BK5 with G in every layout and factor count of make_bk5_G
    (include/bk_harness.h:217-244), with both kernel shapes."""
    E = 7
    nq, _, dbasis, g6i, u = random_case(5, p, E)
    G = oracle.make_bk5_G(g6i, E, nq, nfactors, layout)
    kern = bklib.KERNEL_SWEEP if kernel == "sweep" else bklib.KERNEL_COLUMN
    if engine == "fp32":
        dt, prec, eng, tol = "f32", bklib.PREC_FP32, 0, TOL32
        f = lambda a: a.astype(np.float32).astype(np.float64)
        ref = oracle.bk5(nq, E, dbasis, f(g6i), f(u))
    else:
        dt, prec, tol = "f64", bklib.PREC_FP64, TOL64
        eng = bklib.ENGINE_DFMA if engine == "dfma" else bklib.ENGINE_FF
        ref = oracle.bk5(nq, E, dbasis, g6i, u)
    gu, gg = dev(u, dt), dev(G, dt)
    out = torch.full_like(gu, float("nan"))
    bklib.bk5_apply(p, E, dbasis, gg, gu, out, prec=prec, engine=eng, layout=layout, nfactors=nfactors, kernel=kern)
    torch.cuda.synchronize()
    assert oracle.rel_maxdiff(host(out), ref) < tol


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_bk5_kernel_shapes_agree(bklib, p, prec):
    """The sweep and column kernels give the same operator."""
    E = 37
    nq, _, dbasis, g, u = random_case(5, p, E, seed=99)
    pr = bklib.PREC_FP64 if prec == "fp64" else bklib.PREC_MIXED
    dt = "f64" if prec == "fp64" else "f32"
    gu, gg = dev(u, dt), dev(g, dt)
    outs = []
    for kern in (bklib.KERNEL_SWEEP, bklib.KERNEL_COLUMN):
        out = torch.full_like(gu, float("nan"))
        bklib.bk5_apply(p, E, dbasis, gg, gu, out, prec=pr, kernel=kern)
        outs.append(host(out))
    torch.cuda.synchronize()
    assert oracle.rel_maxdiff(outs[1], outs[0]) < (TOL64 if prec == "fp64" else TOL32)


@pytest.mark.parametrize("p", [2, 5, 8])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_bk5_helmholtz_mass(bklib, p, prec):
    E = 9
    nq, _, dbasis, g, u = random_case(5, p, E)
    mass = np.random.default_rng(p).uniform(0.5, 1.5, E * nq ** 3)
    pr = bklib.PREC_FP64 if prec == "fp64" else bklib.PREC_MIXED
    out = gpu_apply(bklib, 5, p, E, None, dbasis, g, u, pr, mass=mass, lam=1.0)
    if pr == bklib.PREC_FP64:
        ref = oracle.bk5(nq, E, dbasis, g, u, mass=mass, lam=1.0)
        tol = TOL64
    else:
        f = lambda a: a.astype(np.float32).astype(np.float64)
        ref = oracle.bk5(nq, E, dbasis, f(g), f(u), mass=f(mass), lam=1.0)
        tol = TOL32
    assert oracle.rel_maxdiff(out, ref) < tol


@pytest.mark.parametrize("p", [1, 4, 6, 8])
@pytest.mark.parametrize("engine", ["dfma", "ff"])
def test_bk3_coefficient(bklib, p, engine):
    E = 5
    nq, basis, dbasis, g, u = random_case(3, p, E)
    k = np.exp(np.random.default_rng(p).normal(0, 0.5, E * nq ** 3))
    eng = bklib.ENGINE_DFMA if engine == "dfma" else bklib.ENGINE_FF
    out = gpu_apply(bklib, 3, p, E, basis, dbasis, g, u, bklib.PREC_FP64, engine=eng, k=k)
    ref = oracle.bk3(nq, E, basis, dbasis, g, u, k=k)
    assert oracle.rel_maxdiff(out, ref) < TOL64


def test_offset_views(bklib):
    """Arrays that start inside an allocation (16-byte aligned views)."""
    p, E = 7, 6
    nq, _, dbasis, g, u = random_case(5, p, E)
    big_u = dev(np.concatenate([np.zeros(2), u]), "f64")[2:]
    big_g = dev(np.concatenate([np.zeros(2), g]), "f64")[2:]
    out = torch.full((E * nq ** 3 + 2,), float("nan"), dtype=torch.float64, device="cuda")[2:]
    bklib.bk5_apply(p, E, dbasis, big_g, big_u, out)
    torch.cuda.synchronize()
    assert oracle.rel_maxdiff(host(out), oracle.bk5(nq, E, dbasis, g, u)) < TOL64
    # a view one double in is not 16-byte aligned: rejected before any launch
    with pytest.raises(bklib.BKError, match="misaligned"):
        bklib.bk5_apply(p, E - 1, dbasis, big_g, big_u[1:], out)


def test_bounded_wait_timeout(bklib):
    """A device-side wait that nothing completes gives up within its limit,
    records BK_ERR_TIMEOUT, and the context stays usable."""
    L = bklib.lib()
    assert bklib.device_status(reset=True) == bklib.BK_OK
    assert L.bk_set_wait_limit(20000) == 0
    try:
        s = torch.cuda.current_stream().cuda_stream
        assert L.bk_test_wait_timeout(s) == 0
        torch.cuda.synchronize()
        assert bklib.device_status(reset=True) == bklib.BK_ERR_TIMEOUT
    finally:
        assert L.bk_set_wait_limit(0) == 0
    # the next apply runs normally
    p, E = 3, 4
    nq, _, dbasis, g, u = random_case(5, p, E)
    out = gpu_apply(bklib, 5, p, E, None, dbasis, g, u, bklib.PREC_FP64)
    assert oracle.rel_maxdiff(out, oracle.bk5(nq, E, dbasis, g, u)) < TOL64
    assert bklib.device_status(reset=True) == bklib.BK_OK


@pytest.mark.parametrize("p", P_ALL)
@pytest.mark.parametrize("engine", ["dfma", "ff", "fp32", "mixed"])
def test_bk5_gll_even_odd(bklib, p, engine):
    """With the GLL derivative matrix (centro-antisymmetric) BK5 takes the
    even-odd contractions; same operator as the oracle's plain sums."""
    E = 11
    nq = p + 1
    D, _, _ = bklib.bk5_matrices(p)
    rng = np.random.default_rng(100 + p)
    u = rng.uniform(-1, 1, E * nq ** 3)
    g = rng.uniform(0.5, 1.5, E * 6 * nq ** 3)
    if engine in ("dfma", "ff"):
        eng = bklib.ENGINE_DFMA if engine == "dfma" else bklib.ENGINE_FF
        out = gpu_apply(bklib, 5, p, E, None, D, g, u, bklib.PREC_FP64, engine=eng)
        ref = oracle.bk5(nq, E, D, g, u)
        tol = TOL64
    else:
        pr = bklib.PREC_FP32 if engine == "fp32" else bklib.PREC_MIXED
        out = gpu_apply(bklib, 5, p, E, None, D, g, u, pr)
        f = lambda a: a.astype(np.float32).astype(np.float64)
        ref = oracle.bk5(nq, E, D, f(g), f(u))
        tol = TOL32
    assert oracle.rel_maxdiff(out, ref) < tol


@pytest.mark.parametrize("p", P_ALL)
@pytest.mark.parametrize("engine", ["dfma", "ff", "fp32", "mixed"])
@pytest.mark.parametrize("coef", [False, True])
def test_bk3_gll_gauss_even_odd(bklib, p, engine, coef):
    """With GLL nodes and Gauss points (B centro-symmetric, D
    centro-antisymmetric) BK3 takes the even-odd contractions, rectangular
    for the interpolation; same operator as the oracle's plain sums."""
    E = 9
    B, D, _, _, _ = bklib.bk1_bk3_matrices(p)
    nq = p + 2
    rng = np.random.default_rng(200 + p)
    u = rng.uniform(-1, 1, E * (nq - 1) ** 3)
    g = rng.uniform(0.5, 1.5, E * 6 * nq ** 3)
    k = np.exp(rng.normal(0, 0.5, E * nq ** 3)) if coef else None
    if engine in ("dfma", "ff"):
        eng = bklib.ENGINE_DFMA if engine == "dfma" else bklib.ENGINE_FF
        out = gpu_apply(bklib, 3, p, E, B, D, g, u, bklib.PREC_FP64, engine=eng, k=k)
        ref = oracle.bk3(nq, E, B, D, g, u, k=k)
        tol = TOL64
    else:
        pr = bklib.PREC_FP32 if engine == "fp32" else bklib.PREC_MIXED
        out = gpu_apply(bklib, 3, p, E, B, D, g, u, pr, k=k)
        f = lambda a: None if a is None else a.astype(np.float32).astype(np.float64)
        ref = oracle.bk3(nq, E, B, D, f(g), f(u), k=f(k))
        tol = TOL32
    assert np.all(np.isfinite(out))
    assert oracle.rel_maxdiff(out, ref) < tol


@pytest.mark.parametrize("p", P_ALL)
@pytest.mark.parametrize("engine", ["dfma", "ff", "fp32", "mixed"])
def test_bk1_gll_gauss_even_odd(bklib, p, engine):
    """With GLL nodes and Gauss points (B centro-symmetric) BK1 takes the
    even-odd interpolation sweeps; same operator as the oracle's sums."""
    E = 10
    B, _, _, _, _ = bklib.bk1_bk3_matrices(p)
    nq = p + 2
    rng = np.random.default_rng(300 + p)
    u = rng.uniform(-1, 1, E * (nq - 1) ** 3)
    jxw = rng.uniform(0.5, 1.5, E * nq ** 3)
    if engine in ("dfma", "ff"):
        eng = bklib.ENGINE_DFMA if engine == "dfma" else bklib.ENGINE_FF
        out = gpu_apply(bklib, 1, p, E, B, None, jxw, u, bklib.PREC_FP64, engine=eng)
        ref = oracle.bk1(nq, E, B, jxw, u)
        tol = TOL64
    else:
        pr = bklib.PREC_FP32 if engine == "fp32" else bklib.PREC_MIXED
        out = gpu_apply(bklib, 1, p, E, B, None, jxw, u, pr)
        f = lambda a: a.astype(np.float32).astype(np.float64)
        ref = oracle.bk1(nq, E, B, f(jxw), f(u))
        tol = TOL32
    assert np.all(np.isfinite(out))
    assert oracle.rel_maxdiff(out, ref) < tol


@pytest.mark.parametrize("p", P_ALL)
@pytest.mark.parametrize("layout", [0, 1, 2])
@pytest.mark.parametrize("with_mass", [False, True])
def test_bk5_split_g_is_bitwise(bklib, p, layout, with_mass):
    """G split once into float-float pairs (bk_g_to_ff) gives bitwise the
    apply on the doubles: the pairs are the engine's own split of each value.
    The conversion also runs in place."""
    E = 13
    nq = p + 1
    D, _, _ = bklib.bk5_matrices(p)
    rng = np.random.default_rng(300 + p)
    u = dev(rng.uniform(-1, 1, E * nq ** 3), "f64")
    g = dev(rng.uniform(0.5, 1.5, E * 6 * nq ** 3) * (1 + 1e-9 * rng.standard_normal(E * 6 * nq ** 3)), "f64")
    mass = dev(rng.uniform(0.5, 1.5, E * nq ** 3), "f64") if with_mass else None
    v0 = torch.empty_like(u)
    v1 = torch.full_like(u, float("nan"))
    bklib.bk5_apply(p, E, D, g, u, v0, layout=layout, mass=mass, lam=0.7 if with_mass else 0.0)
    gff = bklib.g_to_ff(g)
    bklib.bk5_apply(p, E, D, gff, u, v1, layout=layout, mass=mass, lam=0.7 if with_mass else 0.0,
                    gform=bklib.G_FF)
    g_in_place = g.clone()
    bklib.g_to_ff(g_in_place, out=g_in_place)
    torch.cuda.synchronize()
    assert torch.equal(v0, v1)
    assert torch.equal(g_in_place, gff)
    # hi + lo is the double to 2^-48
    pairs = gff.view(torch.float32).view(-1, 2).double()
    assert torch.max(torch.abs(pairs[:, 0] + pairs[:, 1] - g) / torch.abs(g)).item() < 2.0 ** -47


def test_bk5_split_g_unsupported(bklib):
    """The split G form is for the float-float engine's even-odd sweep kernel
    only: every other combination is rejected, none computes."""
    p, E = 4, 3
    nq = p + 1
    D, _, _ = bklib.bk5_matrices(p)
    g = torch.ones(E * 6 * nq ** 3, dtype=torch.float64, device="cuda")
    u = torch.ones(E * nq ** 3, dtype=torch.float64, device="cuda")
    v = torch.empty_like(u)
    for kw in (dict(engine=bklib.ENGINE_DFMA), dict(prec=bklib.PREC_MIXED), dict(nfactors=9),
               dict(kernel=bklib.KERNEL_COLUMN)):
        with pytest.raises(bklib.BKError, match="precision"):
            bklib.bk5_apply(p, E, D, g, u, v, gform=bklib.G_FF, **kw)
    # a D that is not centro-antisymmetric has no even-odd form
    Dn = np.random.default_rng(1).uniform(-1, 1, (nq, nq))
    with pytest.raises(bklib.BKError, match="precision"):
        bklib.bk5_apply(p, E, Dn, g, u, v, gform=bklib.G_FF)


@pytest.mark.parametrize("p", P_ALL)
@pytest.mark.parametrize("coef", [False, True])
def test_bk3_split_g_is_bitwise(bklib, p, coef):
    """BK3 on G split once into float-float pairs gives bitwise the apply on
    the doubles (GLL nodes, Gauss points: the even-odd path)."""
    E = 7
    B, D, _, _, _ = bklib.bk1_bk3_matrices(p)
    nq = p + 2
    rng = np.random.default_rng(400 + p)
    u = dev(rng.uniform(-1, 1, E * (nq - 1) ** 3), "f64")
    g = dev(rng.uniform(0.5, 1.5, E * 6 * nq ** 3) * (1 + 1e-9 * rng.standard_normal(E * 6 * nq ** 3)), "f64")
    k = dev(np.exp(rng.normal(0, 0.5, E * nq ** 3)), "f64") if coef else None
    v0 = torch.empty_like(u)
    v1 = torch.full_like(u, float("nan"))
    bklib.bk3_apply(p, E, B, D, g, u, v0, k=k)
    bklib.bk3_apply(p, E, B, D, bklib.g_to_ff(g), u, v1, k=k, gform=bklib.G_FF)
    torch.cuda.synchronize()
    assert torch.equal(v0, v1)
    with pytest.raises(bklib.BKError, match="precision"):
        bklib.bk3_apply(p, E, B, D, g, u, v1, prec=bklib.PREC_MIXED, gform=bklib.G_FF)


@pytest.mark.parametrize("p", [1, 3, 6, 7, 8])
@pytest.mark.parametrize("nfactors", [6, 9])
@pytest.mark.parametrize("layout", [0, 1, 2])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_bk5_make_g_matches_oracle(bklib, p, nfactors, layout, prec):
    """The device make_bk5_G is a permutation (and, for 9 factors, a
    duplication) of G6i: bitwise the oracle's restatement of
    include/bk_harness.h:220-244."""
    E = 5
    q = p + 1
    g6i = np.random.default_rng(500 + p).uniform(-1, 1, E * 6 * q ** 3)
    ref = oracle.make_bk5_G(g6i, E, q, nfactors, layout)
    src = dev(g6i, prec)
    out = bklib.bk5_make_g(p, E, src, nfactors=nfactors, layout=layout)
    torch.cuda.synchronize()
    want = ref if prec == "f64" else ref.astype(np.float32).astype(np.float64)
    assert np.array_equal(host(out), want)


def test_bk5_make_g_feeds_the_apply(bklib):
    """G6i relaid on the device to each layout, 6 and 9 factors: the BK5
    apply agrees with the oracle on the interleaved G6."""
    p, E = 7, 6
    q = p + 1
    D, _, _ = bklib.bk5_matrices(p)
    rng = np.random.default_rng(9)
    u = rng.uniform(-1, 1, E * q ** 3)
    g6i = rng.uniform(0.5, 1.5, E * 6 * q ** 3)
    ref = oracle.bk5(q, E, D, g6i, u)
    for nf in (6, 9):
        for layout in (0, 1, 2):
            G = bklib.bk5_make_g(p, E, dev(g6i, "f64"), nfactors=nf, layout=layout)
            v = torch.empty(E * q ** 3, dtype=torch.float64, device="cuda")
            bklib.bk5_apply(p, E, D, G, dev(u, "f64"), v, layout=layout, nfactors=nf)
            torch.cuda.synchronize()
            assert oracle.rel_maxdiff(host(v), ref) < TOL64, (nf, layout)


@pytest.mark.parametrize("p", [1, 2, 3, 5, 8])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_bk1_transpose_jxw_matches_oracle(bklib, p, prec):
    """The device transpose_jxw is bitwise the oracle's restatement of
    include/bk_harness.h:89-102 (JxW(e,p,q,r) -> JxW_t(e,r,q,p))."""
    E = 7
    q = p + 2
    jxw = np.random.default_rng(700 + p).uniform(0.5, 1.5, E * q ** 3)
    if prec == "f32":
        jxw = jxw.astype(np.float32).astype(np.float64)
    out = bklib.bk1_transpose_jxw(p, E, dev(jxw, prec))
    torch.cuda.synchronize()
    assert np.array_equal(host(out), oracle.transpose_jxw(jxw, E, q))


@pytest.mark.parametrize("p", [1, 3, 4, 6, 8])
@pytest.mark.parametrize("prec", [0, 1, 2])
@pytest.mark.parametrize("basis", ["gll", "test"])
def test_bk1_transposed_jxw_apply(bklib, p, prec, basis):
    """BK1 on JxW_t(e,r,q,p) (jxw_layout RQP, the layout of the SYCL BK1
    variants, sycl/bk1_sycl.cpp:74-98) gives bitwise the apply on JxW(e,p,q,r)
    for every engine, on the even-odd (GLL/Gauss) and the plain (test basis)
    paths, and agrees with the oracle."""
    E = 37
    q, P = p + 2, p + 1
    if basis == "gll":
        B = bklib.bk1_bk3_matrices(p)[0]
    else:
        B = oracle.test_basis(P, q)
    rng = np.random.default_rng(40 + p)
    u = rng.uniform(-1, 1, E * P ** 3)
    jxw = rng.uniform(0.5, 1.5, E * q ** 3)
    dt = "f64" if prec == bklib.PREC_FP64 else "f32"
    du, dj = dev(u, dt), dev(jxw, dt)
    djt = bklib.bk1_transpose_jxw(p, E, dj)
    v0 = torch.full_like(du, float("nan"))
    v1 = torch.full_like(du, float("nan"))
    bklib.bk1_apply(p, E, B, dj, du, v0, prec=prec)
    bklib.bk1_apply(p, E, B, djt, du, v1, prec=prec, jxw_layout=bklib.JXW_RQP)
    torch.cuda.synchronize()
    assert torch.equal(v0, v1)
    tol = TOL64 if prec == bklib.PREC_FP64 else 1e-5
    assert oracle.rel_maxdiff(host(v1), oracle.bk1(q, E, B, jxw, u)) < tol


@pytest.mark.parametrize("p", [4, 7])
@pytest.mark.parametrize("h", [1.0 / 64, 1.0 / 16])
def test_bk5_fp64_smooth_field(bklib, p, h):
    """The FP64 forms on a smooth field, u = sin(pi x) sin(pi y) sin(pi z)
    at the nodes of the jittered trilinear mesh: the operator's image
    cancels (v is a second difference, |v| ~ h^2 |u| ... h |u|), which
    amplifies the float-float engine's 2^-48 rounding of the terms; measured
    3e-13 to 4e-13 at p = 7 (DFMA 1e-14), still inside the 1e-12 bound."""
    import math
    Q, E, n = p + 1, 1024, 256
    D, x, w = bklib.bk5_matrices(p)
    G = torch.empty(E * 6 * Q ** 3, dtype=torch.float64, device="cuda")
    X = torch.empty(E * Q ** 3 * 3, dtype=torch.float64, device="cuda")
    bklib.geom_trilinear(Q, E, 16, 16, x, w, 2, h, 0.15, G=G, layout=bklib.LAYOUT_COLUMN, coords=X)
    xyz = X.view(-1, 3)
    u = (torch.sin(math.pi * xyz[:, 0]) * torch.sin(math.pi * xyz[:, 1]) * torch.sin(math.pi * xyz[:, 2])).contiguous()
    g = host(G[: n * 6 * Q ** 3]).reshape(n, 6, Q, Q, Q).transpose(0, 3, 4, 1, 2).copy().ravel()
    ref = oracle.bk5(Q, n, np.asarray(D), g, host(u[: n * Q ** 3]))
    for eng in (bklib.ENGINE_FF, bklib.ENGINE_DFMA):
        v = torch.full_like(u, float("nan"))
        bklib.bk5_apply(p, E, D, G, u, v, prec=bklib.PREC_FP64, engine=eng, layout=bklib.LAYOUT_COLUMN)
        torch.cuda.synchronize()
        assert oracle.rel_maxdiff(host(v[: n * Q ** 3]), ref) < TOL64, (eng, p, h)
