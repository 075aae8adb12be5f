"""Test configuration: the `gpu` marker and the import of the library's Python binding.

The package directory is ``gpu-nurbs_gb300/`` (not an importable identifier); it is loaded
here under the module name ``gpu_nurbs_gb300``.
"""
import glob
import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
PKG_DIR = os.path.join(ROOT, "gpu-nurbs_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _load_pkg():
    if "gpu_nurbs_gb300" in sys.modules:
        return sys.modules["gpu_nurbs_gb300"]
    spec = importlib.util.spec_from_file_location("gpu_nurbs_gb300", os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["gpu_nurbs_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


_load_pkg()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def golden_files():
    return sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(path):
    z = np.load(path, allow_pickle=False)
    d = {k: z[k] for k in z.files}
    for k in ("p", "q", "nu", "nv"):
        if k in d:
            d[k] = int(d[k])
    return d


@pytest.fixture(scope="session")
def nurbs():
    """The binding with the library built (nvcc is available on build hosts)."""
    mod = sys.modules["gpu_nurbs_gb300"]
    if not os.path.exists(mod.LIB_PATH):
        from importlib import util
        spec = util.spec_from_file_location("gn_build", os.path.join(PKG_DIR, "build.py"))
        b = util.module_from_spec(spec)
        spec.loader.exec_module(b)
        b.build()
    return mod
