"""Shared-memory wavefront model of the sweep kernels' work boxes, and the
search that chose their strides (the tables bk5_box and bk3_box in
csrc/bk_kernels.cuh).

A work box holds one element's values at i * PS + j * ZP + k (row stride ZP,
plane stride PS) and consecutive elements ES values apart.  The kernels walk
the box in a few fixed ways, 32 consecutive work items per warp:

  dense      (i, j, k), k fastest: the load of u, the last pass, the store;
  pointwise  G's (k, i, j) order (BK5 layout 2) or the dense order (BK3);
  sweeps     one thread per line of a direction, all lines of the block's
             elements in turn; each reads its NI inputs and writes its NO
             outputs at base + n * stride;
  line passes  (BK5 without direction groups, op 52) the load of u and the
             last pass by i lines (thread per (e, j, k), one access per i)
             and the pointwise stage by k lines (thread per (e, i, j), one
             access per k): a warp's 32 lines span elements where the flat
             walks' 32 points span planes.

A warp instruction on 4-byte values costs the largest number of distinct
words any of the 32 banks is asked for; on 8-byte values each half warp is
one pass over 16 bank pairs.  The score of a box is the weighted mean of
wavefronts per access over the walks of one batch, divided by the
conflict-free count (1 for 4-byte values, 2 for full 8-byte warps): 1.0 is
conflict-free.  For small Q a warp spans several elements, so the element
stride ES matters as much as ZP and PS.

A warp's 128-bit access is four passes of 8 lanes, each one wavefront
when its lanes' 16-byte groups fall in distinct quarters of the 128-byte
bank window.  Op 32 scores BK3's fused flow (op 31) at Q = 8, 4-byte values,
on a box whose rows swap their two 16-byte halves when bit 2 of j is set
(k ^ 4) and whose k lines are 128-bit accesses (WBox3's swizzled form).

    python -m omp_bk_gb300.box_model --op 5 --vbytes 4        # search, prints the table rows
    python -m omp_bk_gb300.box_model --op 32                  # the swizzled Q = 8 box
"""
from __future__ import annotations

import argparse


def wavefronts(addrs, vbytes: int) -> int:
    """Wavefronts of one warp access to the value indices `addrs` (None =
    inactive lane)."""
    if vbytes == 4:
        banks: dict = {}
        for a in addrs:
            if a is not None:
                banks.setdefault(a % 32, set()).add(a)
        return max((len(s) for s in banks.values()), default=0)
    total = 0
    for half in (addrs[:16], addrs[16:]):
        banks = {}
        for a in half:
            if a is not None:
                banks.setdefault(a % 16, set()).add(a)
        total += max((len(s) for s in banks.values()), default=0)
    return total


def _warps(n: int, f):
    return [[f(w) if w < n else None for w in range(w0, w0 + 32)] for w0 in range(0, n, 32)]


def _dense(X, Y, Z, eb, zp, ps, es):
    n = X * Y * Z

    def f(w):
        e, x = divmod(w, n)
        i, r = divmod(x, Y * Z)
        j, k = divmod(r, Z)
        return e * es + i * ps + j * zp + k
    return _warps(eb * n, f)


def _kij(Q, eb, zp, ps, es):
    def f(w):
        e, x = divmod(w, Q ** 3)
        k, r = divmod(x, Q * Q)
        i, j = divmod(r, Q)
        return e * es + i * ps + j * zp + k
    return _warps(eb * Q ** 3, f)


def _sweep(X, Y, Z, d, NO, eb, zp, ps, es, reads=True, writes=True, nread=None):
    """Accesses of a sweep along direction d of an (X, Y, Z) box into extent
    NO (the line enumeration of sweep / sweep_eo / sweep_eor): the NI reads
    and the NO writes of every line (or only one side, or nread reads)."""
    NI = (X, Y, Z)[d]
    LB = Y if d == 2 else Z
    L = X * Y * Z // NI
    sd = ps if d == 0 else (zp if d == 1 else 1)
    out = []
    idx = (list(range(nread if nread is not None else NI)) if reads else []) + (list(range(NO)) if writes else [])
    for n in idx:
        def f(w, n=n):
            e, l = divmod(w, L)
            a, b = divmod(l, LB)
            base = (a * zp + b) if d == 0 else ((a * ps + b) if d == 1 else (a * ps + b * zp))
            return e * es + base + n * sd
        out += _warps(eb * L, f)
    return out


def _lines(Q, eb, zp, ps, es, along):
    """A pass by lines along i (along = 0: thread per (e, j, k)) or along k
    (along = 2: thread per (e, i, j)), one warp access per point of the
    line."""
    out = []
    for n in range(Q):
        def f(w, n=n):
            e, r = divmod(w, Q * Q)
            a, b = divmod(r, Q)
            return e * es + (n * ps + a * zp + b if along == 0 else a * ps + b * zp + n)
        out += _warps(eb * Q * Q, f)
    return out


def walks(op: int, Q: int, eb: int, zp: int, ps: int, es: int):
    """(weight, warps) of one batch of eb elements.  op 5: BK5 (Q points);
    op 3: BK3 (P = Q - 1 nodes, Q points); op 31: BK3's flow fused along k
    for the FP32-storage forms; op 51: BK5 with the fused k-direction last
    pass."""
    if op == 5:
        yield 4, _dense(Q, Q, Q, eb, zp, ps, es)         # load u, last pass (3 reads)
        yield 6, _kij(Q, eb, zp, ps, es)                 # pointwise: 3 reads, 3 writes
        for d in range(3):                               # gradient and transposed
            yield 1, _sweep(Q, Q, Q, d, Q, eb, zp, ps, es)
            yield 1, _sweep(Q, Q, Q, d, Q, eb, zp, ps, es)
        return
    if op == 51:
        # BK5 with the k-direction last pass fused (KFUSE): the transposed
        # k sweep and the dense last pass become one k-line pass reading
        # the three terms
        yield 1, _dense(Q, Q, Q, eb, zp, ps, es)         # load u
        yield 6, _kij(Q, eb, zp, ps, es)                 # pointwise
        for d in range(3):                               # gradient
            yield 1, _sweep(Q, Q, Q, d, Q, eb, zp, ps, es)
        for d in (0, 1):                                 # transposed i, j
            yield 1, _sweep(Q, Q, Q, d, Q, eb, zp, ps, es)
        yield 3, _sweep(Q, Q, Q, 2, Q, eb, zp, ps, es, writes=False)   # last pass: three k lines read
        return
    if op == 52:
        # BK5 FP32 storage (no direction groups): the per-point passes by
        # lines; the k-direction last pass fused (KFUSE) except at Q = 8
        kfuse = Q != 8
        yield 1, _lines(Q, eb, zp, ps, es, 0)           # load u
        yield 6, _lines(Q, eb, zp, ps, es, 2)           # pointwise
        for d in range(3):                              # gradient
            yield 1, _sweep(Q, Q, Q, d, Q, eb, zp, ps, es)
        for d in ((0, 1) if kfuse else (0, 1, 2)):      # transposed
            yield 1, _sweep(Q, Q, Q, d, Q, eb, zp, ps, es)
        if kfuse:                                       # last pass: three k lines read
            yield 3, _sweep(Q, Q, Q, 2, Q, eb, zp, ps, es, writes=False)
        else:                                           # last pass by i lines
            yield 3, _lines(Q, eb, zp, ps, es, 0)
        return
    P = Q - 1
    if op == 3:
        yield 2, _dense(P, P, P, eb, zp, ps, es)         # load u, store v
        for _ in range(2):                               # interpolation and its transpose
            yield 1, _sweep(P, P, P, 0, Q, eb, zp, ps, es)
            yield 1, _sweep(Q, P, P, 1, Q, eb, zp, ps, es)
            yield 1, _sweep(Q, Q, P, 2, Q, eb, zp, ps, es)
        for d in range(3):
            yield 2, _sweep(Q, Q, Q, d, Q, eb, zp, ps, es)
        yield 6, _dense(Q, Q, Q, eb, zp, ps, es)         # pointwise
        return
    # op 31: BK3's even-odd flow fused along k, u and v straight from/to the
    # stage and HBM (the FP32-storage forms)
    yield 1, _sweep(P, P, P, 0, Q, eb, zp, ps, es, reads=False)          # first interpolation: writes
    yield 1, _sweep(Q, P, P, 1, Q, eb, zp, ps, es)                       # second
    yield 1, _sweep(Q, Q, P, 2, Q, eb, zp, ps, es, writes=False)         # k line: P reads
    yield 2, _sweep(Q, Q, Q, 2, Q, eb, zp, ps, es, reads=False)          # ... u and qt written
    for d in (0, 1):                                                     # gradient, transposed
        yield 1, _sweep(Q, Q, Q, d, Q, eb, zp, ps, es)
        yield 1, _sweep(Q, Q, Q, d, Q, eb, zp, ps, es)
    yield 6, _dense(Q, Q, Q, eb, zp, ps, es)                             # pointwise
    yield 3, _sweep(Q, Q, Q, 2, Q, eb, zp, ps, es, writes=False)         # k line: three terms read
    yield 1, _sweep(Q, Q, P, 2, P, eb, zp, ps, es, reads=False)          # ... P written
    yield 1, _sweep(Q, Q, P, 1, P, eb, zp, ps, es)                       # back along j
    yield 1, _sweep(Q, P, P, 0, P, eb, zp, ps, es, writes=False)         # back along i: reads


def wavefronts128(addrs) -> int:
    """Wavefronts of one warp's 128-bit access at the (16-byte aligned)
    4-byte value indices `addrs`: four passes of 8 lanes."""
    total = 0
    for ph in range(4):
        groups: dict = {}
        for a in addrs[8 * ph:8 * ph + 8]:
            if a is not None:
                groups.setdefault((a // 4) % 8, set()).add(a)
        total += max((len(s) for s in groups.values()), default=0)
    return total


def swizzled_at(zp: int, ps: int, es: int, x: int, sb: int):
    """Value index of (e, i, j, k) in a box whose rows have k ^ x when bit
    sb of j is set."""
    def at(e, i, j, k):
        return e * es + i * ps + j * zp + (k ^ (x if (j >> sb) & 1 else 0))
    return at


def _line_walk(at, X, Y, Z, d, NO, eb, reads=True, writes=True, vec=False):
    """(wavefronts, conflict-free count, instructions) of a sweep along d
    through the box addressed by `at`; vec: 128-bit accesses along k."""
    NI = (X, Y, Z)[d]
    LB = Y if d == 2 else Z
    L = X * Y * Z // NI
    step = 4 if vec else 1
    idx = (list(range(0, NI, step)) if reads else []) + (list(range(0, NO, step)) if writes else [])
    wf = ideal = ins = 0
    for n in idx:
        def f(w, n=n):
            e, l = divmod(w, L)
            a, b = divmod(l, LB)
            return at(e, n, a, b) if d == 0 else (at(e, a, n, b) if d == 1 else at(e, a, b, n))
        for ws in _warps(eb * L, f):
            wf += wavefronts128(ws) if vec else wavefronts(ws, 4)
            ideal += 4 if vec else 1
            ins += 1
    return wf, ideal, ins


def score32(zp: int = 8, ps: int = 72, es: int = 576, x: int = 4, sb: int = 2, vec: bool = True, eb: int = 1):
    """Op 31's walks at Q = 8 on the swizzled box with 128-bit k lines:
    (score, wavefronts, conflict-free wavefronts, shared instructions) of
    one element."""
    Q, P = 8, 7
    at = swizzled_at(zp, ps, es, x, sb)

    def dense(X, Y, Z):
        n = X * Y * Z

        def f(w):
            e, r = divmod(w, n)
            i, r = divmod(r, Y * Z)
            j, k = divmod(r, Z)
            return at(e, i, j, k)
        ws = _warps(eb * n, f)
        return sum(wavefronts(a, 4) for a in ws), len(ws), len(ws)

    parts = [
        (1, _line_walk(at, P, P, P, 0, Q, eb, reads=False)),
        (1, _line_walk(at, Q, P, P, 1, Q, eb)),
        (1, _line_walk(at, Q, Q, P, 2, Q, eb, writes=False, vec=vec)),
        (2, _line_walk(at, Q, Q, Q, 2, Q, eb, reads=False, vec=vec)),
        (2, _line_walk(at, Q, Q, Q, 0, Q, eb)),
        (2, _line_walk(at, Q, Q, Q, 1, Q, eb)),
        (6, dense(Q, Q, Q)),
        (3, _line_walk(at, Q, Q, Q, 2, Q, eb, writes=False, vec=vec)),
        (1, _line_walk(at, Q, Q, P, 2, P, eb, reads=False, vec=vec)),
        (1, _line_walk(at, Q, Q, P, 1, P, eb)),
        (1, _line_walk(at, Q, P, P, 0, P, eb, writes=False)),
    ]
    wf = sum(w * p[0] for w, p in parts)
    ideal = sum(w * p[1] for w, p in parts)
    ins = sum(w * p[2] for w, p in parts)
    return wf / ideal, wf, ideal, ins


def score(op: int, Q: int, eb: int, vbytes: int, zp: int, ps: int, es: int) -> float:
    ideal = 1 if vbytes == 4 else 2
    tot = norm = 0.0
    for wgt, ws in walks(op, Q, eb, zp, ps, es):
        for a in ws:
            act = sum(x is not None for x in a)
            if act == 0:
                continue
            tot += wgt * wavefronts(a, vbytes)
            norm += wgt * (ideal if (vbytes == 4 or act > 16) else 1)
    return tot / norm


def legacy(Q: int, vbytes: int):
    """The first strides (ZP, PS, ES): odd rows, plane stride 8 mod 16 / 32."""
    zp = Q + 1 if Q % 2 == 0 else Q
    if vbytes == 8:
        ps = Q * zp if (Q * zp) % 16 == 8 else Q * zp + ((24 - (Q * zp) % 16) % 16)
    else:
        ps = Q * zp if (Q * zp) % 32 == 8 else Q * zp + ((40 - (Q * zp) % 32) % 32)
    return zp, ps, Q * ps


# elements per block that occur (sweep kernel tables and the Helmholtz tiles)
EBS = {
    (5, 4): {2: [12], 3: [12, 17], 4: [8, 10], 5: [4, 6], 6: [3, 4], 7: [2, 3], 8: [1, 2], 9: [1]},
    (5, 8): {2: [16], 3: [16, 14], 4: [8], 5: [4, 5], 6: [4, 3], 7: [2], 8: [2, 1], 9: [3, 1]},
    (3, 4): {3: [16], 4: [8], 5: [6], 6: [4], 7: [3], 8: [1], 9: [1], 10: [1]},
    (3, 8): {3: [12], 4: [8], 5: [8], 6: [3], 7: [3], 8: [1], 9: [3], 10: [1]},
    (31, 4): {3: [16], 4: [8], 5: [6], 6: [4], 7: [3], 8: [1], 9: [1], 10: [1]},
    (51, 4): {2: [12], 3: [12, 14], 4: [8, 8], 5: [4, 5], 6: [3, 3], 7: [2, 2], 9: [1, 1]},
    # the single-order sweep kernels' batches and the Helmholtz launch's
    # tuned tiles (q = 3..9: 42, 16, 10, 3, 2, 2, 1 elements)
    (52, 4): {2: [12], 3: [12, 42], 4: [8, 16], 5: [4, 10], 6: [3], 7: [2], 8: [1, 2], 9: [1]},
}


def mean_score(op, Q, vbytes, zp, ps, es):
    ebs = EBS[(op, vbytes)][Q]
    return sum(score(op, Q, eb, vbytes, zp, ps, es) for eb in ebs) / len(ebs)


def search(op: int, Q: int, vbytes: int):
    """The strides with the lowest mean score (ties: the smaller box)."""
    best = None
    for zp in range(Q, Q + 4):
        for ps in range(Q * zp, Q * zp + 33):
            for pad in range(0, 33):
                s = round(mean_score(op, Q, vbytes, zp, ps, Q * ps + pad), 3)
                key = (s, Q * ps + pad)
                if best is None or key < best[0]:
                    best = (key, zp, ps, Q * ps + pad)
    return best[1], best[2], best[3], best[0][0]


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--op", type=int, choices=(3, 5, 31, 32, 51, 52), default=5)
    ap.add_argument("--vbytes", type=int, choices=(4, 8), default=4)
    args = ap.parse_args(argv)
    if args.op == 32:
        s, wf, ideal, ins = score32()
        s0, wf0, ideal0, ins0 = score32(8, 71, 568, 0, 2, vec=False)
        print(f"Q=8 swizzled {{8, 72, 576}}, 128-bit k lines: score {s:.2f}, {wf} wavefronts, "
              f"{ins} instructions per element ({{8, 71, 568}} unswizzled: {s0:.2f}, {wf0}, {ins0})")
        return
    for Q in sorted(EBS[(args.op, args.vbytes)]):
        zp, ps, es, s = search(args.op, Q, args.vbytes)
        lz, lp, le = legacy(Q, args.vbytes)
        print(f"Q={Q}: {{{zp}, {ps}, {es}}}  score {s:.2f}  (first strides {lz},{lp},{le}: "
              f"{mean_score(args.op, Q, args.vbytes, lz, lp, le):.2f})", flush=True)


if __name__ == "__main__":
    main()
