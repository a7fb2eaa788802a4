"""The work-box stride tables of the sweep kernels (csrc/bk_kernels.cuh)
against the shared-memory wavefront model that chose them
(omp_bk_gb300/box_model.py): every entry is a valid box (rows, planes and
elements do not overlap) and scores no worse than the first, odd-row
strides.  No GPU."""
import os
import re

import pytest

from omp_bk_gb300 import box_model

SRC = os.path.join(os.path.dirname(__file__), "..", "omp_bk_gb300", "csrc", "bk_kernels.cuh")


def _table(name):
    text = open(SRC).read()
    m = re.search(r"constexpr int " + name + r"\[\d+\]\[3\] = \{(.*?)\};", text, re.S)
    assert m, name
    return [tuple(int(x) for x in t) for t in re.findall(r"\{\s*(\d+),\s*(\d+),\s*(\d+)\s*\}", m.group(1))]


@pytest.mark.parametrize("op,name,vb,q0", [(52, "t4", 4, 2), (5, "t8", 8, 2), (3, "b4", 4, 3), (3, "b8", 8, 3)])
def test_tables_valid_and_no_worse(op, name, vb, q0):
    rows = _table(name)
    qs = sorted(box_model.EBS[(op, vb)])
    assert len(rows) == len(qs) and qs[0] == q0
    for Q, (zp, ps, es) in zip(qs, rows):
        assert zp >= Q and (Q - 1) * zp + Q <= ps and Q * ps <= es, (Q, zp, ps, es)
        new = box_model.mean_score(op, Q, vb, zp, ps, es)
        old = box_model.mean_score(op, Q, vb, *box_model.legacy(Q, vb))
        assert new <= old + 1e-9, (Q, new, old)


def test_wavefront_counts():
    # 32 consecutive 4-byte words: one wavefront; all lanes on one bank: 32
    assert box_model.wavefronts(list(range(32)), 4) == 1
    assert box_model.wavefronts([32 * i for i in range(32)], 4) == 32
    # a broadcast is one wavefront
    assert box_model.wavefronts([5] * 32, 4) == 1
    # 8-byte values: two half-warp passes when conflict-free
    assert box_model.wavefronts(list(range(32)), 8) == 2


def test_swizzled_q8_box():
    # op 32's scalar, unswizzled form is op 31 itself; the swizzled box with
    # 128-bit k lines (WBox3<8, float, true>) has fewer wavefronts and fewer
    # shared-memory instructions
    s0, wf0, ideal0, ins0 = box_model.score32(8, 71, 568, 0, 2, vec=False)
    assert abs(s0 - box_model.score(31, 8, 1, 4, 8, 71, 568)) < 1e-12
    s, wf, ideal, ins = box_model.score32()
    assert (wf, ins) == (474, 344) and (wf0, ins0) == (612, 424)
    # the swizzle permutes each row: every (i, j, k) of an element has its
    # own slot inside the element's 576 values
    at = box_model.swizzled_at(8, 72, 576, 4, 2)
    slots = {at(0, i, j, k) for i in range(8) for j in range(8) for k in range(8)}
    assert len(slots) == 512 and min(slots) >= 0 and max(slots) < 576


def test_swizzled_box_constants_match_the_model():
    # the kernel header's swizzled BK3 box is the one op 32 scores
    text = open(SRC).read()
    assert re.search(r"constexpr int bk3_swz\(int q, int vbytes\) \{ return \(q == 8 && vbytes == 4\) \? 4 : 0; \}", text)
    assert "static constexpr int SB = 2;" in text
    for name, val in (("ZP", 8), ("PS", 72), ("size", 576)):
        assert re.search(r"static constexpr int " + name + r" = X \? " + str(val) + r" :", text), name


def test_two_base_line_addressing():
    # BoxLine's per-line bases (two per line, picked by the compile-time
    # index) give the swizzled address of every value of every line, and a
    # k line's two 16-byte halves start at la(0) and la(4)
    zp, ps, es, x, sb = 8, 72, 576, 4, 2
    at = box_model.swizzled_at(zp, ps, es, x, sb)
    swz = lambda j: x if (j >> sb) & 1 else 0

    def line(d, e, a, b):
        eb = e * es
        if d == 0:
            b0 = eb + a * zp + (b ^ swz(a))
            return lambda n: b0 + n * ps
        if d == 1:
            b0, b1 = eb + a * ps + b, eb + a * ps + (b ^ x)
            return lambda n: (b1 if (n >> sb) & 1 else b0) + n * zp
        m = swz(b)
        b0, b1 = eb + a * ps + b * zp + m, eb + a * ps + b * zp - m
        return lambda n: (b1 if n & x else b0) + n

    for e in range(2):
        for i in range(8):
            for j in range(8):
                for k in range(8):
                    want = at(e, i, j, k)
                    assert line(0, e, j, k)(i) == want
                    assert line(1, e, i, k)(j) == want
                    assert line(2, e, i, j)(k) == want
                la = line(2, e, i, j)
                for c in (0, 4):
                    assert la(c) % 4 == 0 and [la(c) + q for q in range(4)] == [at(e, i, j, c + q) for q in range(4)]


def test_line_walks_table():
    """The 4-byte BK5 box serves the line walks of the FP32-storage sweep
    body (op 52): the entries re-searched for them (q = 2, 4) score below
    the boxes they replaced, and a line pass touches every point of a batch
    exactly once."""
    t4 = dict(zip(sorted(box_model.EBS[(52, 4)]), _table("t4")))
    assert t4[4] == (4, 19, 80) and t4[2] == (2, 15, 36)
    assert box_model.mean_score(52, 4, 4, *t4[4]) < box_model.mean_score(52, 4, 4, 6, 24, 97)
    assert box_model.mean_score(52, 2, 4, *t4[2]) < box_model.mean_score(52, 2, 4, 2, 16, 36)
    for Q, eb in ((3, 12), (4, 8), (8, 2)):
        zp, ps, es = t4[Q]
        for along in (0, 2):
            seen = [a for ws in box_model._lines(Q, eb, zp, ps, es, along) for a in ws if a is not None]
            want = {e * es + i * ps + j * zp + k for e in range(eb) for i in range(Q) for j in range(Q)
                    for k in range(Q)}
            assert len(seen) == eb * Q ** 3 and set(seen) == want, (Q, along)
