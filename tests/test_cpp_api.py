"""The C++ classes of include/gpu_nurbs.hpp (NuFile, Surface, Pool, Graph, Server): a program
using all of them (tests/cpp_api_check.cpp) compiles and links against the library here, and
on the GPU it recovers the parameters of points evaluated on a patch to 1e-9."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp_api_check.cpp")


@pytest.fixture(scope="module")
def cpp_exe(nurbs, tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    libdir = os.path.dirname(nurbs.LIB_PATH)
    exe = str(tmp_path_factory.mktemp("cppapi") / "cpp_api_check")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(cuda, "include"), SRC, "-o", exe, "-L" + libdir, "-lgpunurbs",
           "-Wl,-rpath," + libdir, "-L" + os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def test_cpp_classes_compile_and_link(cpp_exe):
    assert os.access(cpp_exe, os.X_OK)


@pytest.mark.gpu
def test_cpp_classes_round_trip_on_gpu(cpp_exe):
    r = subprocess.run([cpp_exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
