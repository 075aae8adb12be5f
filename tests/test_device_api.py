"""The header-only device API (include/gpu_nurbs_device.cuh) under the reference's names:
findSpan, MatrixNPosition, MatrixSurfacePoint, MatrixSurfaceDerivative{U,V,UU,UV,VV}.

A helper (tests/device_api_check.cu) walks each golden (u, v) the way the reference's
EvaluateRandom does and must reproduce the reference's S and derivatives bit for bit: on the
host here (no GPU needed) and in a CUDA kernel on the GPU."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_files, load_golden

SRC = os.path.join(ROOT, "tests", "device_api_check.cu")
MODEL_FILES = [f for f in golden_files() if os.path.basename(f).startswith(("model_", "synth_"))
               and "eval" in np.load(f).files]
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


@pytest.fixture(scope="module")
def dapi(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out = str(tmp_path_factory.mktemp("dapi") / "libdapi.so")
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-shared",
           "-Xcompiler", "-fPIC,-ffp-contract=off", "-o", out, SRC]
    subprocess.run(cmd, check=True, capture_output=True)
    L = C.CDLL(out)
    L.dapi_eval_host.restype = C.c_int
    L.dapi_eval_host.argtypes = [C.c_int] * 4 + [_dp, _dp, _dp, _dp, C.c_longlong, _dp]
    L.dapi_eval_device.restype = C.c_int
    L.dapi_eval_device.argtypes = [C.c_int] * 4 + [_dp, _dp, _dp, C.c_longlong, _dp, C.c_longlong, _dp]
    return L


def _args(g):
    f = lambda x: np.ascontiguousarray(x, dtype=np.float64)
    return g["p"], g["q"], g["nu"], g["nv"], f(g["knots_u"]), f(g["knots_v"]), f(g["matrix_n"]), f(g["uv"])


@pytest.mark.parametrize("path", MODEL_FILES, ids=lambda p: os.path.basename(p)[:-4])
def test_device_api_host_bit_exact(dapi, path):
    g = load_golden(path)
    p, q, nu, nv, ku, kv, M, uv = _args(g)
    out = np.empty((18, len(uv)), dtype=np.float64)
    assert dapi.dapi_eval_host(p, q, nu, nv, ku, kv, M, uv, len(uv), out) == 0
    assert np.array_equal(out, g["eval"], equal_nan=True)


@pytest.mark.gpu
@pytest.mark.parametrize("path", MODEL_FILES, ids=lambda p: os.path.basename(p)[:-4])
def test_device_api_kernel_bit_exact(dapi, path):
    g = load_golden(path)
    p, q, nu, nv, ku, kv, M, uv = _args(g)
    out = np.empty((18, len(uv)), dtype=np.float64)
    assert dapi.dapi_eval_device(p, q, nu, nv, ku, kv, M, len(M), uv, len(uv), out) == 0
    assert np.array_equal(out, g["eval"], equal_nan=True)
