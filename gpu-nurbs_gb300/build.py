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
import hashlib
import json
import os
import platform
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
EXACT_TUS = {"k_convert.cu", "k_tree.cu", "k_legacy.cu", "k_quadtree.cu"}
EXPLICIT_FMA_TUS = {"k_eval.cu", "k_invert.cu", "k_pool.cu", "k_pcurve.cu", "k_project.cu"}
SOURCES = ["k_convert.cu", "k_tree.cu", "k_legacy.cu", "k_eval.cu", "k_invert.cu", "api.cpp", "nu_io.cpp", "k_probe.cu", "k_static.cu", "k_pool.cu", "pool.cpp", "server.cpp", "k_pcurve.cu", "k_project.cu", "k_quadtree.cu"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _digest(parts, files) -> str:
    """Content hash of a build step: its command line, the host machine and its input files."""
    h = hashlib.sha256()
    h.update(platform.machine().encode())
    for x in parts:
        h.update(x.encode() + b"\0")
    for f in files:
        with open(f, "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()


def _fresh(out: str, digest: str) -> bool:
    """An output is reused only when its stamp records the same content hash (sources, flags,
    machine): modification times are not trusted, since copied trees carry arbitrary ones."""
    stamp = out + ".stamp"
    if not (os.path.exists(out) and os.path.exists(stamp)):
        return False
    with open(stamp) as f:
        return f.read().strip() == digest


def _stamp(out: str, digest: str):
    with open(out + ".stamp", "w") as f:
        f.write(digest + "\n")


def _compile(src: str, verbose: bool):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    deps = [path] + sorted(os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh")))
    deps.append(os.path.join(INCLUDE, "gpu_nurbs.h"))
    cmd = [nvcc()] + ARCH + COMMON
    if src in EXACT_TUS or src in EXPLICIT_FMA_TUS:
        cmd.append("--fmad=false")
    if src.endswith(".cpp"):
        cmd += ["-x", "cu"]
    digest = _digest(cmd + [src], deps)
    if _fresh(obj, digest):
        return obj, False
    if verbose:
        cmd += ["-Xptxas", "-v"]
    cmd += ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    _stamp(obj, digest)
    return obj, True


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compiles what changed and links the library.  Writes _build/build_record.json: which
    translation units were compiled in this call and which were reused (same content hash)."""
    os.makedirs(OBJ, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        res = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [o for o, _ in res]
    link_cmd = [nvcc()] + ARCH + ["-shared"] + [os.path.basename(o) for o in objs] + ["-lcudart"]
    digest = _digest(link_cmd, objs)
    linked = not _fresh(LIB, digest)
    if linked:
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
        _stamp(LIB, digest)
    with open(os.path.join(OBJ, "build_record.json"), "w") as f:
        json.dump({"machine": platform.machine(), "compiled": [s for s, (_, c) in zip(SOURCES, res) if c],
                   "reused": [s for s, (_, c) in zip(SOURCES, res) if not c], "linked": linked}, f)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
