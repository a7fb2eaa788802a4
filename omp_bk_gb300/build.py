"""Build the CUDA library of omp_bk_gb300 in place (nvcc, sm_103a only).

    python -m omp_bk_gb300.build          # or omp_bk_gb300.build.build()

Produces omp_bk_gb300/_lib/libbk_gb300.so from csrc/ (one object per
translation unit and engine, compiled in parallel) and the C++ host driver
omp_bk_gb300/_lib/bk_cuda.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
OBJDIR = os.path.join(ROOT, "_build", "obj")
LIB = os.path.join(LIBDIR, "libbk_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags() -> list[str]:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-Wall",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "--expt-relaxed-constexpr", "-diag-suppress", "177"]


def _units() -> list[tuple[str, list[str], str]]:
    """(source, extra flags, object) of every translation unit."""
    u = []
    for eng in range(4):
        for op in (1, 3, 7):
            u.append(("bk_ops.cu", [f"-DBK_ENGINE_TU={eng}", f"-DBK_OP_TU={op}"], f"bk_ops_{eng}_{op}.o"))
        for op in (5, 6):
            for lay in range(3):
                u.append(("bk_ops.cu", [f"-DBK_ENGINE_TU={eng}", f"-DBK_OP_TU={op}", f"-DBK_LAYOUT_TU={lay}"],
                          f"bk_ops_{eng}_{op}_{lay}.o"))
    for src in ("bk_helmholtz.cu", "bk_api.cu", "bk_geom.cu", "bk_basis.cpp", "bk_vec.cu", "bk_noalloc.cu", "bk_host.cu",
                "bk_probe.cu"):
        u.append((src, [], src.rsplit(".", 1)[0] + ".o"))
    return u


def _compile(src: str, extra: list[str], obj: str, verbose: bool) -> str:
    out = os.path.join(OBJDIR, obj)
    srcp = os.path.join(CSRC, src)
    deps = [srcp] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps += [os.path.join(ROOT, "include", h) for h in os.listdir(os.path.join(ROOT, "include"))]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cmd = [nvcc()] + _flags() + extra + ["-c", srcp, "-o", out]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src} {extra}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stderr.strip()):
        print(r.stderr, file=sys.stderr)
    return out


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile every CUDA translation unit for sm_103a and link the library.
    Returns the library path."""
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    units = sorted(_units(), key=lambda t: not ("_6_" in t[2] or "_5_" in t[2]))
    jobs = jobs or min(len(units), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda t: _compile(t[0], t[1], t[2], verbose), units))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-cudart", "static"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    _driver(verbose)
    return LIB


DRIVER = os.path.join(LIBDIR, "bk_cuda")


def _driver(verbose: bool) -> None:
    """The C++ host driver with the reference drivers' command line, linked
    against the library (rpath $ORIGIN)."""
    src = os.path.join(CSRC, "driver", "bk_driver.cpp")
    if os.path.exists(DRIVER) and os.path.getmtime(DRIVER) >= max(os.path.getmtime(src), os.path.getmtime(LIB)):
        return
    cmd = [nvcc()] + ARCH + ["-O2", "-std=c++17", "-Xcompiler", "-fopenmp,-Wall", "-I" + os.path.join(ROOT, "include"),
                             src, "-o", DRIVER, "-L" + LIBDIR, "-lbk_gb300", "-Xlinker", "-rpath,$ORIGIN",
                             "-Xcompiler", "-fopenmp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    print(build(verbose=True))
