"""Generate tests/golden/golden.npz from the reference's OWN host kernels.

Run where the reference's sources are present (the tree named by
$BK_REF_DIR or --ref; by default the one oracle/Makefile names):
``make -C oracle ref`` compiles them by include path into
oracle/_ref/, and this script calls them through ctypes.  The fixtures pin the
oracle (tests/test_oracle.py) and the CUDA kernels (tests/test_golden_gpu.py)
to the reference's results on the reference's own test data:

  * random data: fill_random_test_data's LCG, seed 12345 (include/bk_common.h:92-107),
    in ~ [-1,1], JxW/G ~ 1.5 + [-1,1], test basis cos(a*cols+b) (:63-86);
    bk::SumFactorization<double, nq> of BK1, BK3, BK5 for p = 1..8 on E_RAND
    elements, and the harness references reference_bk1/3/5 (float inputs);
  * constant data of the drivers (openmp/BK1.cpp:40-44, BK3.cpp:56-60,
    BK5.cpp:118-120): in = 3, JxW = 1, G = 2, the driver's "norm =" line for
    float (the drivers' precision) and double on E_CONST elements;
  * make_bk5_G in every (F, layout) and transpose_jxw on one element;
  * the first LCG draws and a test basis.

Usage:  python tests/golden/make_golden.py [--ref <reference tree>]
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
E_RAND = 2
E_CONST = 64
SEED = 12345

dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def load(ref):
    cmd = ["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"] + ([f"REF={ref}"] if ref else [])
    subprocess.run(cmd, check=True)
    d = os.path.join(ROOT, "oracle", "_ref")
    L = {k: C.CDLL(os.path.join(d, f"libbkref_{k}.so")) for k in ("bk1", "bk3", "bk5", "harness")}
    for sfx, p in (("f64", dp), ("f32", fp)):
        f = getattr(L["bk1"], "bkref_bk1_" + sfx); f.restype = C.c_int; f.argtypes = [C.c_int, C.c_size_t, p, p, p, p]
        f = getattr(L["bk3"], "bkref_bk3_" + sfx); f.restype = C.c_int; f.argtypes = [C.c_int, C.c_size_t, p, p, p, p, p]
        f = getattr(L["bk5"], "bkref_bk5_" + sfx); f.restype = C.c_int; f.argtypes = [C.c_int, C.c_size_t, p, p, p, p]
    H = L["harness"]
    H.bkref_reference_bk1.argtypes = [C.c_int, C.c_size_t, fp, fp, fp, dp]
    H.bkref_reference_bk3.argtypes = [C.c_int, C.c_size_t, fp, fp, fp, fp, dp]
    H.bkref_reference_bk5.argtypes = [C.c_int, C.c_size_t, fp, fp, fp, dp]
    H.bkref_make_bk5_G.argtypes = [fp, C.c_size_t, C.c_int, C.c_int, C.c_int, fp]
    H.bkref_transpose_jxw.argtypes = [fp, C.c_size_t, C.c_int, fp]
    H.bkref_fill_random_f64.argtypes = [dp, C.c_size_t, dp, C.c_size_t, C.c_uint32]
    H.bkref_make_test_basis_f64.argtypes = [C.c_int, C.c_int, dp]
    H.bkref_make_test_basis_f32.argtypes = [C.c_int, C.c_int, fp]
    H.bkref_norm2_f64.restype = C.c_double; H.bkref_norm2_f64.argtypes = [dp, C.c_size_t]
    H.bkref_norm2_f32.restype = C.c_double; H.bkref_norm2_f32.argtypes = [fp, C.c_size_t]
    return L


def basis(H, rows, cols, dt):
    m = np.empty(rows * cols, dtype=dt)
    (H.bkref_make_test_basis_f32 if dt == np.float32 else H.bkref_make_test_basis_f64)(rows, cols, m)
    return m


def rand(H, nin, nj):
    a = np.empty(nin); b = np.empty(nj)
    H.bkref_fill_random_f64(a, nin, b, nj, SEED)
    return a, b


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("BK_REF_DIR"),
                    help="the reference's source tree (default: $BK_REF_DIR, else the oracle Makefile's)")
    args = ap.parse_args()
    L = load(args.ref)
    H = L["harness"]
    out = {}
    norms = {}
    for p in range(1, 9):
        # BK1 and BK3: nq = p + 2, nm = p + 1; BK5: nq = p + 1
        for bk in (1, 3, 5):
            nq = p + 1 if bk == 5 else p + 2
            nm = nq if bk == 5 else nq - 1
            nin = nm ** 3
            ngeo = nq ** 3 if bk == 1 else 6 * nq ** 3
            # random data, double
            u, g = rand(H, E_RAND * nin, E_RAND * ngeo)
            o = np.empty(E_RAND * nin)
            if bk == 1:
                rc = L["bk1"].bkref_bk1_f64(p, E_RAND, basis(H, nm, nq, np.float64), g, u, o)
            elif bk == 3:
                rc = L["bk3"].bkref_bk3_f64(p, E_RAND, basis(H, nm, nq, np.float64),
                                            basis(H, nq, nq, np.float64), g, u, o)
            else:
                rc = L["bk5"].bkref_bk5_f64(p, E_RAND, basis(H, nq, nq, np.float64), g, u, o)
            assert rc == 0
            out[f"bk{bk}_p{p}_rand_f64"] = o
            # harness reference: float inputs, double arithmetic
            uf, gf = u.astype(np.float32), g.astype(np.float32)
            r = np.empty(E_RAND * nin)
            if bk == 1:
                H.bkref_reference_bk1(nq, E_RAND, basis(H, nm, nq, np.float32), gf, uf, r)
            elif bk == 3:
                H.bkref_reference_bk3(nq, E_RAND, basis(H, nm, nq, np.float32), basis(H, nq, nq, np.float32), gf, uf, r)
            else:
                H.bkref_reference_bk5(nq, E_RAND, basis(H, nq, nq, np.float32), gf, uf, r)
            out[f"bk{bk}_p{p}_harness"] = r
            # constant data of the drivers, float and double
            for dt, sfx in ((np.float32, "f32"), (np.float64, "f64")):
                u = np.full(E_CONST * nin, 3.0, dtype=dt)
                g = np.full(E_CONST * ngeo, 1.0 if bk == 1 else 2.0, dtype=dt)
                o = np.empty(E_CONST * nin, dtype=dt)
                if bk == 1:
                    rc = getattr(L["bk1"], "bkref_bk1_" + sfx)(p, E_CONST, basis(H, nm, nq, dt), g, u, o)
                elif bk == 3:
                    rc = getattr(L["bk3"], "bkref_bk3_" + sfx)(p, E_CONST, basis(H, nm, nq, dt), basis(H, nq, nq, dt), g, u, o)
                else:
                    rc = getattr(L["bk5"], "bkref_bk5_" + sfx)(p, E_CONST, basis(H, nq, nq, dt), g, u, o)
                assert rc == 0
                nrm = (H.bkref_norm2_f32 if dt == np.float32 else H.bkref_norm2_f64)(o, o.size)
                norms[f"bk{bk}_p{p}_const_{sfx}"] = nrm
                # first element's output, the driver's constant-data known answer per point
                out[f"bk{bk}_p{p}_const_{sfx}_e0"] = o[:nin].astype(np.float64)
    # layouts
    nq = 3
    g6i = rand(H, 0, 6 * nq ** 3)[1].astype(np.float32)
    for F in (6, 9):
        for layout in (0, 1, 2):
            G = np.empty(F * nq ** 3, dtype=np.float32)
            H.bkref_make_bk5_G(g6i, 1, nq, F, layout, G)
            out[f"make_bk5_G_nq3_F{F}_L{layout}"] = G.astype(np.float64)
    jx = rand(H, 0, 4 ** 3)[1].astype(np.float32)
    t = np.empty(4 ** 3, dtype=np.float32)
    H.bkref_transpose_jxw(jx, 1, 4, t)
    out["transpose_jxw_nq4"] = t.astype(np.float64)
    out["lcg_first_32"] = rand(H, 32, 0)[0]
    out["test_basis_4x5_f64"] = basis(H, 4, 5, np.float64)
    out["test_basis_4x5_f32"] = basis(H, 4, 5, np.float32).astype(np.float64)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    meta = {"generator": "tests/golden/make_golden.py", "seed": SEED, "E_rand": E_RAND,
            "E_const": E_CONST, "norms": norms}
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print(f"wrote {len(out)} arrays, {len(norms)} norms")


if __name__ == "__main__":
    sys.exit(main())
