"""The C++ driver with the reference drivers' command line
(omp_bk_gb300/_lib/bk_cuda BK1|BK3|BK5 <p> [nelmt] [ntests]): its result
lines, the constant-data "norm =" known answers of the reference's own
drivers (tests/golden/golden.json, the same E = 64 elements) and its
BK_CHECK host comparison, for every variant it offers."""
import os
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "omp_bk_gb300", "_lib", "bk_cuda")


def _run(op, p, nelmt, prec, kernels, check=True):
    env = dict(os.environ, BK_PREC=prec, BK_KERNEL=kernels)
    if check:
        env["BK_CHECK"] = "1"
    r = subprocess.run([DRIVER, op, str(p), str(nelmt), "2"], env=env, capture_output=True, text=True, timeout=300)
    return r.returncode, r.stdout + r.stderr


@pytest.mark.parametrize("bk", [1, 3, 5])
@pytest.mark.parametrize("p", [2, 5, 7])
def test_driver_known_answers_and_check(golden, bk, p):
    _, meta = golden
    E = meta["E_const"]
    # the driver prints the norm with 10 significant digits, as the
    # reference's drivers do: FP64 agrees to that precision
    for prec, kernels, tol in (("fp32", "fp32 mixed", 2e-5), ("fp64", "ff dfma", 1e-9)):
        rc, out = _run(f"BK{bk}", p, E, prec, kernels)
        assert rc == 0, out
        assert "FAIL" not in out, out
        rates = re.findall(r"^(\w+)\s+SumFactorization -> nelmt = (\d+) GDoF/s = (\S+) GB/s = (\S+)", out, re.M)
        assert {r[0] for r in rates} == set(kernels.split()), out
        assert all(int(r[1]) == E and float(r[2]) > 0 for r in rates)
        ref = meta["norms"][f"bk{bk}_p{p}_const_{'f32' if prec == 'fp32' else 'f64'}"]
        for name, nrm in re.findall(r"^(\w+)\s+norm = (\S+)", out, re.M):
            assert abs(float(nrm) - ref) <= tol * abs(ref), (name, nrm, ref)


def test_driver_rejects_unsupported_order():
    rc, out = _run("BK5", 9, 8, "fp64", "ff", check=False)
    assert rc != 0 and "unsupported polynomial order" in out


def test_driver_random_data_check():
    env = dict(os.environ, BK_PREC="fp64", BK_KERNEL="ff dfma", BK_CHECK="1", BK_RANDOM="1")
    r = subprocess.run([DRIVER, "BK3", "6", "37", "2"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "FAIL" not in r.stdout, r.stdout + r.stderr
    assert len(re.findall(r"relerr = (\S+)", r.stdout)) == 2


def _run_ff(p, nelmt, extra=None):
    env = dict(os.environ)
    env.pop("BK_RANDOM", None)
    env.update(extra or {})
    r = subprocess.run([DRIVER, "BK1_ff", str(p), str(nelmt), "2"], env=env, capture_output=True, text=True,
                       timeout=300)
    return r.returncode, r.stdout + r.stderr


@pytest.mark.parametrize("p", [2, 5, 7])
def test_bk1_ff_harness(golden, p):
    """BK1_ff mode (openmp/BK1_ff.cpp): double, float and float-float rows on
    the same data, the double and float-float norms equal to the reference's
    FP64 known answer, the float-float error against double below BK_TOL
    (default 1e-10) with "ok" and exit code 0."""
    _, meta = golden
    E = meta["E_const"]
    rc, out = _run_ff(p, E)
    assert rc == 0, out
    assert re.search(rf"^SumFactorization -> nelmt = {E} nq = {p + 2} data = constant", out, re.M), out
    rows = dict((n, (float(g), float(nrm))) for n, g, nrm in
                re.findall(r"^(double|float-float|float)\s+GDoF/s =\s*(\S+) GB/s =\s*\S+ norm = (\S+)", out, re.M))
    assert set(rows) == {"double", "float", "float-float"}, out
    ref = meta["norms"][f"bk1_p{p}_const_f64"]
    assert abs(rows["double"][1] - ref) <= 1e-9 * abs(ref)
    assert abs(rows["float-float"][1] - ref) <= 1e-9 * abs(ref)
    assert abs(rows["float"][1] - ref) <= 1e-5 * abs(ref)
    m = re.search(r"^ok: float-float rel\. error vs double = (\S+) \(tol = 1e-10\)", out, re.M)
    assert m and float(m.group(1)) <= 1e-10, out
    assert float(re.search(r"^float\s+rel\. error vs double = (\S+)", out, re.M).group(1)) < 1e-5


def test_bk1_ff_random_and_tolerance():
    """BK_RANDOM data passes; a tolerance below the float-float error (set on
    the host, nothing faults) prints FAIL and exits 1."""
    rc, out = _run_ff(3, 300, {"BK_RANDOM": "1"})
    assert rc == 0 and "data = random" in out and re.search(r"^ok: ", out, re.M), out
    rc, out = _run_ff(3, 300, {"BK_RANDOM": "1", "BK_TOL": "1e-30"})
    assert rc == 1 and re.search(r"^FAIL: float-float rel\. error vs double = \S+ \(tol = 1e-30\)", out, re.M), out
