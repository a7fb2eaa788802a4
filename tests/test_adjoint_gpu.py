"""The hand-written BK3 adjoint (dL/dk, dL/dG of L = 1/2 |A(k) u - f|^2) and
the FP64 vector kernels, on the GPU.

  - against the oracle's FP64 host gradient (oracle/bk_oracle.c
    bko_bk3_adjoint): relative max difference < 1e-12;
  - against central finite differences, step h = 1e-6, along 64 seeded
    directions in (k, G) at the full configuration (p = 4, E = 65536,
    log k ~ N(0, 0.5^2), u, f ~ U[-1, 1]): relative error < 1e-7.  The
    difference quotient (L(x + h d) - L(x - h d)) / (2h) is evaluated as
    (r+ - r-) . (r+ + r-) / (4h) with r+- the residuals at x +- h d: the same
    number without the cancellation of two nearly equal sums of squares.
"""
import numpy as np
import pytest
import torch

import oracle
from gpu_util import dev, host

pytestmark = pytest.mark.gpu


def _geom(bk, p, E, seed):
    """BK3 inputs of the configuration: affine mesh G (factor-major) at the
    Gauss points, B and D of order p, on the device."""
    B, D, xq, wq, _ = bk.bk1_bk3_matrices(p)
    Q = p + 2
    G = torch.empty(E * 6 * Q ** 3, dtype=torch.float64, device="cuda")
    bk.geom_affine(Q, E, xq, wq, seed, 1.0 / 16, 0.2, G=G, layout=bk.LAYOUT_FACTOR)
    return B, D, G


@pytest.mark.parametrize("p", [1, 2, 4, 6, 8])
@pytest.mark.parametrize("engine", ["dfma", "ff"])
def test_adjoint_vs_host_gradient(bklib, p, engine):
    bk = bklib
    E = 9
    Q, P = p + 2, p + 1
    B, D, G = _geom(bk, p, E, 11)
    rng = np.random.default_rng(p)
    k = np.exp(rng.normal(0, 0.5, E * Q ** 3))
    u = rng.uniform(-1, 1, E * P ** 3)
    res = rng.uniform(-1, 1, E * P ** 3)
    eng = bk.ENGINE_DFMA if engine == "dfma" else bk.ENGINE_FF
    dk = torch.full((E * Q ** 3,), float("nan"), dtype=torch.float64, device="cuda")
    dG = torch.full((E * 6 * Q ** 3,), float("nan"), dtype=torch.float64, device="cuda")
    bk.bk3_adjoint(p, E, B, D, G, dev(k, "f64"), dev(u, "f64"), dev(res, "f64"), dk, dG, engine=eng)
    torch.cuda.synchronize()
    rk, rG = oracle.bk3_adjoint(Q, E, B, D, host(G), k, u, res)
    assert oracle.rel_maxdiff(host(dk), rk) < 1e-12
    assert oracle.rel_maxdiff(host(dG), rG) < 1e-12


@pytest.mark.parametrize("p", [2, 5])
def test_adjoint_general_bases(bklib, p):
    """Bases without the point symmetry (the plain sweeps, not the even-odd
    ones) against the oracle's host gradient."""
    from gpu_util import random_case
    bk = bklib
    E = 7
    nq, B, D, g, u = random_case(3, p, E)
    rng = np.random.default_rng(50 + p)
    k = np.exp(rng.normal(0, 0.5, E * nq ** 3))
    res = rng.uniform(-1, 1, E * (nq - 1) ** 3)
    dk = torch.full((E * nq ** 3,), float("nan"), dtype=torch.float64, device="cuda")
    dG = torch.full((E * 6 * nq ** 3,), float("nan"), dtype=torch.float64, device="cuda")
    bk.bk3_adjoint(p, E, B, D, dev(g, "f64"), dev(k, "f64"), dev(u, "f64"), dev(res, "f64"), dk, dG)
    torch.cuda.synchronize()
    rk, rG = oracle.bk3_adjoint(nq, E, B, D, g, k, u, res)
    assert oracle.rel_maxdiff(host(dk), rk) < 1e-12
    assert oracle.rel_maxdiff(host(dG), rG) < 1e-12


def test_adjoint_finite_differences_full(bklib):
    """Configuration: BK3 adjoint, FP64, p = 4 (P = 5, Q = 6), E = 65536."""
    bk = bklib
    p, E = 4, 65536
    Q, P = p + 2, p + 1
    B, D, G = _geom(bk, p, E, 21)
    nq, nm = E * Q ** 3, E * P ** 3
    k = bk.fill_lognormal(torch.empty(nq, dtype=torch.float64, device="cuda"), 31, 0.5)
    u = bk.fill_uniform(torch.empty(nm, dtype=torch.float64, device="cuda"), 32)
    f = bk.fill_uniform(torch.empty(nm, dtype=torch.float64, device="cuda"), 33)
    ws = bk.dot_workspace(max(nq * 6, nm))
    out = torch.zeros(1, dtype=torch.float64, device="cuda")

    def residual(kk, GG, r):
        # native FP64 for the difference quotient: a 1e-6 step amplifies the
        # ~1e-14 rounding of the float-float engine to ~1e-7
        bk.bk3_apply(p, E, B, D, GG, u, r, k=kk, engine=bk.ENGINE_DFMA)
        bk.axpby(-1.0, f, 1.0, r)   # r = A u - f
        return r

    r0 = residual(k, G, torch.empty(nm, dtype=torch.float64, device="cuda"))
    dk = torch.empty(nq, dtype=torch.float64, device="cuda")
    dG = torch.empty(6 * nq, dtype=torch.float64, device="cuda")
    bk.bk3_adjoint(p, E, B, D, G, k, u, r0, dk, dG)
    h = 1e-6
    rp = torch.empty_like(r0)
    rm = torch.empty_like(r0)
    kp, km, Gp, Gm = (torch.empty_like(k), torch.empty_like(k), torch.empty_like(G), torch.empty_like(G))
    dkd = torch.empty_like(k)
    dGd = torch.empty_like(G)
    worst = 0.0
    for t in range(64):
        bk.fill_uniform(dkd, 1000 + t)
        bk.fill_uniform(dGd, 2000 + t)
        dGd.mul_(G.abs().mean())   # directions of the size of G
        kp.copy_(k); bk.axpby(h, dkd, 1.0, kp)
        km.copy_(k); bk.axpby(-h, dkd, 1.0, km)
        Gp.copy_(G); bk.axpby(h, dGd, 1.0, Gp)
        Gm.copy_(G); bk.axpby(-h, dGd, 1.0, Gm)
        residual(kp, Gp, rp)
        residual(km, Gm, rm)
        diff = rp - rm
        ssum = rp + rm
        bk.dot(diff, ssum, out, ws)
        fd = out.item() / (4 * h)
        bk.dot(dk, dkd, out, ws)
        an = out.item()
        bk.dot(dG, dGd, out, ws)
        an += out.item()
        worst = max(worst, abs(fd - an) / abs(an))
    assert worst < 1e-7, worst
    # and the FP64 host gradient on a slice of the elements
    Es = 256
    rk, rG = oracle.bk3_adjoint(Q, Es, B, D, host(G)[: Es * 6 * Q ** 3], host(k)[: Es * Q ** 3],
                                host(u)[: Es * P ** 3], host(r0)[: Es * P ** 3])
    assert oracle.rel_maxdiff(host(dk)[: Es * Q ** 3], rk) < 1e-12
    assert oracle.rel_maxdiff(host(dG)[: Es * 6 * Q ** 3], rG) < 1e-12


@pytest.mark.parametrize("n", [1, 7, 1000, 1 << 20, 3_000_001])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_dot_axpby(bklib, n, dtype):
    bk = bklib
    x = bk.fill_uniform(torch.empty(n, dtype=dtype, device="cuda"), 5)
    y = bk.fill_uniform(torch.empty(n, dtype=dtype, device="cuda"), 6)
    ws = bk.dot_workspace(n)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    bk.dot(x, y, out, ws)
    ref = float(np.dot(host(x), host(y)))
    assert abs(out.item() - ref) <= 1e-12 * max(1.0, np.abs(host(x) * host(y)).sum())
    bk.dot(x, x, out, ws, half=True)
    assert abs(out.item() - 0.5 * float(np.dot(host(x), host(x)))) <= 1e-12 * n
    yh = host(y)
    bk.axpby(2.0, x, -0.5, y)
    tol = 1e-15 if dtype == torch.float64 else 1e-6
    assert np.allclose(host(y), 2.0 * host(x) - 0.5 * yh, rtol=0, atol=tol * 4)


def test_stream_kernels(bklib):
    bk = bklib
    n = 1 << 16
    b = bk.fill_uniform(torch.empty(7 * n, dtype=torch.float32, device="cuda"), 1)
    a = torch.empty(n, dtype=torch.float32, device="cuda")
    c = bk.fill_uniform(torch.empty(n, dtype=torch.float32, device="cuda"), 2)
    bk.stream_kernel(bk.STREAM_COPY, a, b[:n])
    assert torch.equal(a, b[:n])
    bk.stream_kernel(bk.STREAM_TRIAD, a, b[:n], c)
    assert torch.allclose(a, b[:n] + 3 * c, rtol=1e-6, atol=1e-6)
    bk.stream_kernel(bk.STREAM_MIX, a, b, reads=7)
    assert torch.allclose(a, b.view(7, n).sum(0), atol=1e-5)


@pytest.mark.parametrize("p", [1, 3, 4, 6, 8])
def test_adjoint_split_g_is_bitwise(bklib, p):
    """The backward kernel on G split once into float-float pairs
    (bk_g_to_ff) gives bitwise the gradients of the double G."""
    bk = bklib
    E = 7
    Q, P = p + 2, p + 1
    B, D, G = _geom(bk, p, E, 13)
    rng = np.random.default_rng(40 + p)
    k = dev(np.exp(rng.normal(0, 0.5, E * Q ** 3)), "f64")
    u = dev(rng.uniform(-1, 1, E * P ** 3), "f64")
    res = dev(rng.uniform(-1, 1, E * P ** 3), "f64")
    dk0, dk1 = (torch.empty(E * Q ** 3, dtype=torch.float64, device="cuda") for _ in range(2))
    dG0, dG1 = (torch.empty(E * 6 * Q ** 3, dtype=torch.float64, device="cuda") for _ in range(2))
    bk.bk3_adjoint(p, E, B, D, G, k, u, res, dk0, dG0)
    bk.bk3_adjoint(p, E, B, D, bk.g_to_ff(G), k, u, res, dk1, dG1, gform=bk.G_FF)
    torch.cuda.synchronize()
    assert torch.equal(dk0, dk1) and torch.equal(dG0, dG1)
    with pytest.raises(bk.BKError, match="precision"):
        bk.bk3_adjoint(p, E, B, D, G, k, u, res, dk1, dG1, engine=bk.ENGINE_DFMA, gform=bk.G_FF)
