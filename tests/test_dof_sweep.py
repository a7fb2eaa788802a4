"""The DoF-sweep harness (throughput versus problem size, the reference's
scripts/study/dof_sweep.sh): element counts, CSV columns, and one small sweep
on the GPU."""
import math

import pytest

from omp_bk_gb300 import dof_sweep


def test_element_counts_log_spaced():
    c = dof_sweep.element_counts(3, 1e3, 1e7, 4)
    assert c == sorted(set(c))
    assert c[0] == round(1e3 / 27) and c[-1] == round(1e7 / 27)
    assert len(c) <= 4 * 4 + 1
    ratios = [b / a for a, b in zip(c, c[1:])]
    assert all(1.5 < r < 2.0 for r in ratios)   # 10^(1/4) = 1.78 apart
    assert dof_sweep.element_counts(9, 1, 10, 1) == [1]


def test_sizes_per_element():
    # BK1 p=3: 64 modes, 125 quadrature values; BK3 p=6: 343 modes, 6 * 512
    assert dof_sweep.values_per_element(1, 3) == (64, 125)
    assert dof_sweep.values_per_element(3, 6) == (343, 3072)
    assert dof_sweep.values_per_element(5, 7) == (512, 3072)
    assert dof_sweep.quad_per_dim(3, 6) == 8 and dof_sweep.quad_per_dim(5, 7) == 8


@pytest.mark.gpu
def test_small_sweep_writes_csv(bklib, tmp_path):
    out = tmp_path / "sweep.csv"
    assert dof_sweep.main(["--bk", "1,3,5", "--p", "2", "--kernels", "ff,mixed", "--dof-min", "1e3",
                           "--dof-max", "1e4", "--ppd", "2", "--ntests", "2", "--out", str(out)]) == 0
    lines = out.read_text().splitlines()
    assert lines[0] == dof_sweep.HEADER
    rows = [ln.split(",") for ln in lines[1:]]
    assert len(rows) == 3 * 2 * len(dof_sweep.element_counts(3, 1e3, 1e4, 2))
    for r in rows:
        assert r[0] == "cuda" and int(r[4]) == int(r[3]) * 27
        assert all(math.isfinite(float(x)) and float(x) > 0 for x in r[5:9])
    stream = (tmp_path / "sweep.csv.stream").read_text()
    assert "copy" in stream and "triad" in stream
