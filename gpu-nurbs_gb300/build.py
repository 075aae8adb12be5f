"""Build recipe for libgpunurbs.so (sm_103a), in place, without cmake.

Each translation unit is compiled by nvcc in parallel, then linked into one shared library
next to this file.  Translation units whose results must be bit-identical to the
reference's unfused FP64 arithmetic (span conversion, subdivision tree, legacy drop-in
kernels) are compiled with --fmad=false.  So are the evaluation and inversion kernels: their
arithmetic writes each fused multiply-add explicitly, and without compiler contraction a
point's result is the same in every kernel that computes it (single surface, pool, graph).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgpunurbs.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC,
          "--expt-relaxed-constexpr", "-Wno-deprecated-gpu-targets"]
EXACT_TUS = {"k_convert.cu", "k_tree.cu", "k_legacy.cu"}
EXPLICIT_FMA_TUS = {"k_eval.cu", "k_invert.cu", "k_pool.cu"}
SOURCES = ["k_convert.cu", "k_tree.cu", "k_legacy.cu", "k_eval.cu", "k_invert.cu", "api.cpp", "nu_io.cpp", "k_probe.cu", "k_static.cu", "k_pool.cu", "pool.cpp", "server.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, verbose: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(INCLUDE, "gpu_nurbs.h"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + ARCH + COMMON
    if src in EXACT_TUS or src in EXPLICIT_FMA_TUS:
        cmd.append("--fmad=false")
    if src.endswith(".cpp"):
        cmd += ["-x", "cu"]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    cmd += ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
