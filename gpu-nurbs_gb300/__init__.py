"""gpu_nurbs_gb300 — Python host binding of the GB300 NURBS engine.

Thin ctypes layer over ``libgpunurbs.so`` (the C-ABI of ``include/gpu_nurbs.h``).  It mirrors
the reference's calls (Qiang-Zou/GPU-NURBS): ``read_nu`` for ``readNu`` (src/main.cu:45-113),
``Surface`` for the GetMatrixN upload (src/NURBS/Evaluate.cu:3-88), ``Surface.eval`` for
MatrixSurfacePoint / MatrixSurfaceDerivative* (Evaluate.cu:159-930), ``Surface.tree`` and
``Surface.candidates`` for the subdivision tree and the NewInverse scan (src/kernel/kernel.cu),
and ``Surface.invert`` for NewInverse + GaussNewton.

Device buffers are torch CUDA tensors (torch is used for device memory and streams only);
all computation happens in the library's CUDA kernels.  There is no CPU fallback: if the
library is missing, importing this module raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgpunurbs.so")

OK = 0
E_INVALID, E_CUDA, E_NOMEM, E_IO, E_PARSE, E_UNSUPPORTED, E_BUDGET, E_TIMEOUT, E_STATE = range(-1, -10, -1)
S, SU, SV, SUU, SUV, SVV = 1, 2, 4, 8, 16, 32
SUUU, SUUV, SUVV, SVVV = 64, 128, 256, 512
N, NU, NV, NUU, NUV, NVV = 1, 2, 4, 8, 16, 32
PREC_FP64, PREC_MIXED, PREC_FP32, PREC_EXACT = 0, 1, 2, 3
PCURVE_JUMP, PCURVE_AMBIGUOUS, PCURVE_NOT_FOUND = 1, 2, 4
INV_FOUND, INV_AMBIGUOUS, INV_NO_CANDIDATE, INV_NOT_CONVERGED = 0, 1, 2, 3
PTR_HOST, PTR_DEVICE = 0, 1
TREE_NODES = 65


class NurbsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{msg} (status {code})")
        self.code = code


class NuDesc(C.Structure):
    _fields_ = [("degree_u", C.c_int), ("degree_v", C.c_int), ("cp_u", C.c_int), ("cp_v", C.c_int),
                ("knots_u", C.POINTER(C.c_double)), ("knots_v", C.POINTER(C.c_double)),
                ("cps", C.POINTER(C.c_double)), ("weights", C.POINTER(C.c_double))]


class SurfaceDesc(C.Structure):
    _fields_ = [("degree_u", C.c_int), ("degree_v", C.c_int), ("cp_u", C.c_int), ("cp_v", C.c_int),
                ("knots_u", C.c_void_p), ("knots_v", C.c_void_p), ("cps", C.c_void_p), ("weights", C.c_void_p)]


class PoolInfo(C.Structure):
    _fields_ = [("budget_bytes", C.c_int64), ("used_bytes", C.c_int64), ("surfaces", C.c_int),
                ("max_surfaces", C.c_int), ("tile_queries", C.c_int), ("ctas_per_sm", C.c_int)]


class SurfaceInfo(C.Structure):
    _fields_ = [("degree_u", C.c_int), ("degree_v", C.c_int), ("cp_u", C.c_int), ("cp_v", C.c_int),
                ("spans_u", C.c_int), ("spans_v", C.c_int), ("device_bytes", C.c_int64), ("tree_built", C.c_int)]


_vp = C.c_void_p
_i64 = C.c_int64

# name -> (restype, argtypes); the list is the C-ABI of include/gpu_nurbs.h
SIGNATURES = {
    "nurbs_status_string": (C.c_char_p, [C.c_int]),
    "nurbs_last_error": (C.c_char_p, []),
    "nurbs_version": (C.c_char_p, []),
    "nurbs_nu_read": (C.c_int, [C.c_char_p, C.POINTER(NuDesc)]),
    "nurbs_nu_parse": (C.c_int, [C.c_char_p, _i64, C.POINTER(NuDesc)]),
    "nurbs_nu_write": (C.c_int, [C.c_char_p, C.POINTER(NuDesc)]),
    "nurbs_nu_free": (None, [C.POINTER(NuDesc)]),
    "nurbs_surface_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, C.c_int, _vp,
                                       C.POINTER(_vp)]),
    "nurbs_surface_destroy": (C.c_int, [_vp]),
    "nurbs_surface_info": (C.c_int, [_vp, C.POINTER(SurfaceInfo)]),
    "nurbs_matrix_n_size": (_i64, [C.c_int, C.c_int, C.c_int, C.c_int]),
    "nurbs_matrix_n_position": (_i64, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "nurbs_get_matrix_n": (C.c_int, [_vp, _vp, _vp]),
    "nurbs_get_matrix_n_raw": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    "nurbs_get_matrix_n_noalloc": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    "nurbs_eval": (C.c_int, [_vp, _vp, _i64, C.c_uint, _vp, C.c_int, _vp]),
    "nurbs_eval_f32": (C.c_int, [_vp, _vp, _i64, C.c_uint, _vp, _vp]),
    "nurbs_evaluate_random": (C.c_int, [_vp, _vp, _i64, _vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp]),
    "nurbs_build_tree": (C.c_int, [_vp, C.c_int, _vp]),
    "nurbs_tree_export": (C.c_int, [_vp, _vp, _vp, _vp]),
    "nurbs_candidates": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp]),
    "nurbs_invert": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp, C.c_int, _vp]),
    "nurbs_invert_host": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp, C.c_int, _vp]),
    "nurbs_invert_count": (C.c_int, [_vp, _vp, _i64, C.c_int, _vp, _vp]),
    "nurbs_pcurve": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp, _vp, C.c_int, _vp]),
    "nurbs_project": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp, C.c_int, _vp]),
    "nurbs_invert_quadtree": (C.c_int, [_vp, _vp, _i64, C.c_double, _vp, _vp, _vp, C.c_int, _vp]),
    "nurbs_normal_cones_export": (C.c_int, [_vp, _vp, _vp, _vp]),
    "nurbs_eval_normal": (C.c_int, [_vp, _vp, _i64, C.c_uint, _vp, _vp]),
    "nurbs_probe_fp_peak": (C.c_int, [C.c_int, C.POINTER(C.c_double), _vp]),
    "nurbs_pool_create": (C.c_int, [_i64, C.c_int, C.POINTER(_vp)]),
    "nurbs_pool_destroy": (C.c_int, [_vp]),
    "nurbs_pool_add": (C.c_int, [_vp, C.c_int, C.POINTER(SurfaceDesc), _vp, _vp]),
    "nurbs_pool_remove": (C.c_int, [_vp, C.c_int, _vp]),
    "nurbs_pool_info": (C.c_int, [_vp, C.POINTER(PoolInfo)]),
    "nurbs_pool_surface_bytes": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, C.POINTER(_i64)]),
    "nurbs_pool_last_error": (C.c_char_p, []),
    "nurbs_pool_set_config": (C.c_int, [_vp, C.c_int, C.c_int]),
    "nurbs_pool_invert": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int, _vp]),
    "nurbs_pool_eval": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _i64, C.c_uint, _vp, _vp]),
    "nurbs_pool_autotune": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int, _i64, C.c_char_p, _vp,
                                      C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_float)]),
    "nurbs_pool_graph_create": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int, C.POINTER(_vp)]),
    "nurbs_graph_launch": (C.c_int, [_vp, _vp]),
    "nurbs_graph_destroy": (C.c_int, [_vp]),
    "nurbs_server_create": (C.c_int, [_vp, _vp, C.POINTER(_vp)]),
    "nurbs_server_destroy": (C.c_int, [_vp]),
    "nurbs_server_submit_invert": (C.c_int, [_vp, C.c_int, _vp, _i64, _vp, _vp, _vp, _vp, C.POINTER(C.c_uint64)]),
    "nurbs_server_submit_upload": (C.c_int, [_vp, C.POINTER(SurfaceDesc), _vp, _vp, C.POINTER(C.c_uint64)]),
    "nurbs_server_wait": (C.c_int, [_vp, C.c_uint64, C.c_int, C.POINTER(C.c_int)]),
    "nurbs_server_poll": (C.c_int, [_vp, _vp, _vp, C.c_int, C.POINTER(C.c_int)]),
    "nurbs_server_drain": (C.c_int, [_vp, C.c_int]),
    "nurbs_server_pause": (C.c_int, [_vp, C.c_int]),
    "nurbs_server_stats": (C.c_int, [_vp, _vp]),
    "nurbs_server_replay": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                      _vp, C.c_int]),
}

_lib = None


def lib():
    """The loaded C-ABI library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libgpunurbs.so not built at {LIB_PATH}; run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int, what: str = ""):
    if rc != OK:
        msg = lib().nurbs_last_error().decode(errors="replace")
        raise NurbsError(rc, f"{what}: {msg or lib().nurbs_status_string(rc).decode()}")


# ------------------------------------------------------------------------ .nu files
def _desc_to_dict(d: NuDesc) -> dict:
    p, q, nu, nv = d.degree_u, d.degree_v, d.cp_u, d.cp_v
    return dict(p=p, q=q, nu=nu, nv=nv,
                knots_u=np.ctypeslib.as_array(d.knots_u, (p + nu + 1,)).copy(),
                knots_v=np.ctypeslib.as_array(d.knots_v, (q + nv + 1,)).copy(),
                cps=np.ctypeslib.as_array(d.cps, (nu * nv * 3,)).copy().reshape(nu * nv, 3),
                weights=np.ctypeslib.as_array(d.weights, (nu * nv,)).copy())


def read_nu(path: str) -> dict:
    """Reads a .nu file with the library's reader (readNu grammar)."""
    d = NuDesc()
    rc = lib().nurbs_nu_read(path.encode(), C.byref(d))
    if rc != OK:
        raise NurbsError(rc, f"nurbs_nu_read({path})")
    try:
        return _desc_to_dict(d)
    finally:
        lib().nurbs_nu_free(C.byref(d))


def parse_nu(text: str) -> dict:
    b = text.encode()
    d = NuDesc()
    rc = lib().nurbs_nu_parse(b, len(b), C.byref(d))
    if rc != OK:
        raise NurbsError(rc, "nurbs_nu_parse")
    try:
        return _desc_to_dict(d)
    finally:
        lib().nurbs_nu_free(C.byref(d))


def write_nu(path: str, surf: dict):
    ku = np.ascontiguousarray(surf["knots_u"], np.float64)
    kv = np.ascontiguousarray(surf["knots_v"], np.float64)
    cps = np.ascontiguousarray(surf["cps"], np.float64).reshape(-1)
    w = np.ascontiguousarray(surf["weights"], np.float64)
    dp = C.POINTER(C.c_double)
    d = NuDesc(int(surf["p"]), int(surf["q"]), int(surf["nu"]), int(surf["nv"]), ku.ctypes.data_as(dp),
               kv.ctypes.data_as(dp), cps.ctypes.data_as(dp), w.ctypes.data_as(dp))
    check(lib().nurbs_nu_write(path.encode(), C.byref(d)), "nurbs_nu_write")


# -------------------------------------------------------------------------- helpers
def _torch():
    import torch
    return torch


def _stream(stream=None):
    if stream is not None:
        return stream
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t) -> int:
    return t.data_ptr()


# -------------------------------------------------------------------------- surface
class Surface:
    """A surface resident on the GPU in matrix form, with its subdivision tree."""

    def __init__(self, surf: dict, stream=None):
        self.p, self.q = int(surf["p"]), int(surf["q"])
        self.nu, self.nv = int(surf["nu"]), int(surf["nv"])
        ku = np.ascontiguousarray(surf["knots_u"], np.float64)
        kv = np.ascontiguousarray(surf["knots_v"], np.float64)
        cps = np.ascontiguousarray(surf["cps"], np.float64).reshape(-1)
        w = np.ascontiguousarray(surf["weights"], np.float64).reshape(-1)
        h = C.c_void_p()
        rc = lib().nurbs_surface_create(self.p, self.q, self.nu, self.nv, ku.ctypes.data, kv.ctypes.data,
                                        cps.ctypes.data, w.ctypes.data, PTR_HOST, _stream(stream), C.byref(h))
        check(rc, "nurbs_surface_create")
        self.h = h
        self.knots_u, self.knots_v = ku, kv

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().nurbs_surface_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> SurfaceInfo:
        i = SurfaceInfo()
        check(lib().nurbs_surface_info(self.h, C.byref(i)), "nurbs_surface_info")
        return i

    def matrix_n(self, stream=None):
        """The span matrices in the reference MatrixN layout (empty spans zero)."""
        torch = _torch()
        n = lib().nurbs_matrix_n_size(self.p, self.q, self.nu, self.nv)
        out = torch.zeros(n, dtype=torch.float64, device="cuda")
        check(lib().nurbs_get_matrix_n(self.h, _ptr(out), _stream(stream)), "nurbs_get_matrix_n")
        return out

    def eval(self, uv, mask: int = S, stream=None, precision: int = PREC_FP64):
        """uv: (n,2) float64 CUDA tensor -> (3*nblocks, n) float64 SoA tensor.  precision
        PREC_EXACT: the reference's FP64 expressions term by term (mask <= 63)."""
        torch = _torch()
        uv = uv.contiguous()
        n = uv.shape[0]
        nb = bin(mask & 1023).count("1")
        out = torch.empty((3 * nb, n), dtype=torch.float64, device=uv.device)
        check(lib().nurbs_eval(self.h, _ptr(uv), n, mask, _ptr(out), precision, _stream(stream)), "nurbs_eval")
        return out

    def eval_normal(self, uv, mask: int = N, stream=None):
        """Normal N = Su x Sv and its derivatives (N, NU, NV, NUU, NUV, NVV bits) at uv ((n,2)
        CUDA tensor) -> (3*nblocks, n) float64 SoA tensor."""
        torch = _torch()
        uv = uv.contiguous()
        n = uv.shape[0]
        nb = bin(mask & 63).count("1")
        out = torch.empty((3 * nb, n), dtype=torch.float64, device=uv.device)
        check(lib().nurbs_eval_normal(self.h, _ptr(uv), n, mask, _ptr(out), _stream(stream)), "nurbs_eval_normal")
        return out

    def eval_f32(self, uv, mask: int = S, stream=None):
        torch = _torch()
        uv = uv.contiguous()
        n = uv.shape[0]
        nb = bin(mask & 1023).count("1")
        out = torch.empty((3 * nb, n), dtype=torch.float32, device=uv.device)
        check(lib().nurbs_eval_f32(self.h, _ptr(uv), n, mask, _ptr(out), _stream(stream)), "nurbs_eval_f32")
        return out

    def tree(self):
        nodes = np.zeros((TREE_NODES, 10), np.float64)
        div = np.zeros(TREE_NODES, np.uint8)
        built = np.zeros(TREE_NODES, np.uint8)
        check(lib().nurbs_tree_export(self.h, nodes.ctypes.data, div.ctypes.data, built.ctypes.data),
              "nurbs_tree_export")
        return nodes, div, built

    def candidates(self, P, stream=None):
        torch = _torch()
        P = P.contiguous()
        n = P.shape[0]
        lst = torch.empty((n, TREE_NODES), dtype=torch.int32, device=P.device)
        cnt = torch.empty(n, dtype=torch.int32, device=P.device)
        check(lib().nurbs_candidates(self.h, _ptr(P), n, _ptr(lst), _ptr(cnt), _stream(stream)), "nurbs_candidates")
        return lst, cnt

    def invert(self, P, precision: int = PREC_MIXED, stream=None, out=None):
        """P: (n,3) float64 CUDA tensor -> (uv (n,2), status (n,), residual (n,))."""
        torch = _torch()
        P = P.contiguous()
        n = P.shape[0]
        if out is None:
            uv = torch.empty((n, 2), dtype=torch.float64, device=P.device)
            st = torch.empty(n, dtype=torch.int32, device=P.device)
            res = torch.empty(n, dtype=torch.float64, device=P.device)
        else:
            uv, st, res = out
        check(lib().nurbs_invert(self.h, _ptr(P), n, _ptr(uv), _ptr(st), _ptr(res), precision, _stream(stream)),
              "nurbs_invert")
        return uv, st, res

    def project(self, P, precision: int = PREC_FP64, stream=None, out=None):
        """Closest point over the closed domain (nurbs_project): P (n,3) float64 CUDA tensor ->
        (uv (n,2), status (n,), residual (n,))."""
        torch = _torch()
        P = P.contiguous()
        n = P.shape[0]
        if out is None:
            uv = torch.empty((n, 2), dtype=torch.float64, device=P.device)
            st = torch.empty(n, dtype=torch.int32, device=P.device)
            res = torch.empty(n, dtype=torch.float64, device=P.device)
        else:
            uv, st, res = out
        check(lib().nurbs_project(self.h, _ptr(P), n, _ptr(uv), _ptr(st), _ptr(res), precision, _stream(stream)),
              "nurbs_project")
        return uv, st, res

    def invert_quadtree(self, P, max_edge: float, precision: int = PREC_FP64, stream=None, out=None):
        """Adaptive quadtree inversion (nurbs_invert_quadtree): P (n,3) float64 CUDA tensor ->
        (uv (n,2), status (n,), residual (n,))."""
        torch = _torch()
        P = P.contiguous()
        n = P.shape[0]
        if out is None:
            uv = torch.empty((n, 2), dtype=torch.float64, device=P.device)
            st = torch.empty(n, dtype=torch.int32, device=P.device)
            res = torch.empty(n, dtype=torch.float64, device=P.device)
        else:
            uv, st, res = out
        check(lib().nurbs_invert_quadtree(self.h, _ptr(P), n, float(max_edge), _ptr(uv), _ptr(st), _ptr(res),
                                          precision, _stream(stream)), "nurbs_invert_quadtree")
        return uv, st, res

    def normal_cones(self):
        """The projection's culling data (nurbs_normal_cones_export): normal boxes (65, 6),
        FP32 records (65, 20), lattice points (65, 81, 3)."""
        nb = np.zeros((TREE_NODES, 6), np.float64)
        cr = np.zeros((TREE_NODES, 20), np.float32)
        lat = np.zeros((TREE_NODES, 81, 3), np.float32)
        check(lib().nurbs_normal_cones_export(self.h, nb.ctypes.data, cr.ctypes.data, lat.ctypes.data),
              "nurbs_normal_cones_export")
        return nb, cr, lat

    def pcurve(self, C, precision: int = PREC_MIXED, stream=None):
        """p-curve of ordered curve samples C ((n,3) CUDA tensor): (uv (n,2), status, residual,
        flags) with flags PCURVE_JUMP / PCURVE_AMBIGUOUS / PCURVE_NOT_FOUND."""
        torch = _torch()
        C = C.contiguous()
        n = C.shape[0]
        uv = torch.empty((n, 2), dtype=torch.float64, device=C.device)
        st = torch.empty(n, dtype=torch.int32, device=C.device)
        res = torch.empty(n, dtype=torch.float64, device=C.device)
        fl = torch.empty(n, dtype=torch.int32, device=C.device)
        check(lib().nurbs_pcurve(self.h, _ptr(C), n, _ptr(uv), _ptr(st), _ptr(res), _ptr(fl), precision,
                                 _stream(stream)), "nurbs_pcurve")
        return uv, st, res, fl

    def count_work(self, P, precision: int = PREC_MIXED, stream=None) -> dict:
        """Work of one inversion of P (CUDA tensor), from the kernel's counting variant:
        seed iterations and final FP64 polishes."""
        P = P.contiguous()
        counts = (C.c_ulonglong * 2)()
        check(lib().nurbs_invert_count(self.h, _ptr(P), P.shape[0], precision, C.cast(counts, C.c_void_p),
                                       _stream(stream)), "nurbs_invert_count")
        return {"seed_iterations": int(counts[0]), "final_polishes": int(counts[1])}

    def invert_host(self, P: np.ndarray, precision: int = PREC_MIXED, stream=None, out=None):
        """Host buffers in and out (copies inside the call)."""
        P = np.ascontiguousarray(P, np.float64).reshape(-1, 3)
        n = P.shape[0]
        if out is None:
            uv = np.empty((n, 2), np.float64)
            st = np.empty(n, np.int32)
            res = np.empty(n, np.float64)
        else:
            uv, st, res = out
        rc = lib().nurbs_invert_host(self.h, P.ctypes.data, n, uv.ctypes.data, st.ctypes.data, res.ctypes.data,
                                     precision, _stream(stream))
        check(rc, "nurbs_invert_host")
        return uv, st, res


def get_matrix_n_raw(p, q, nu, nv, knots_u, knots_v, cps, weights, stream=None):
    """Legacy GetMatrixN with device tensors; returns the MatrixN tensor."""
    torch = _torch()
    n = lib().nurbs_matrix_n_size(p, q, nu, nv)
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    check(lib().nurbs_get_matrix_n_raw(_ptr(out), p, q, nu, nv, _ptr(knots_u), _ptr(knots_v), _ptr(cps),
                                       _ptr(weights), _stream(stream)), "nurbs_get_matrix_n_raw")
    return out


def evaluate_random(uv, matrix_n, p, q, nu, nv, knots_u, knots_v, stream=None):
    """Legacy EvaluateRandom with device tensors; returns (n,3) points."""
    torch = _torch()
    n = uv.shape[0]
    out = torch.empty((n, 3), dtype=torch.float64, device=uv.device)
    check(lib().nurbs_evaluate_random(_ptr(uv), _ptr(out), n, _ptr(matrix_n), p, q, nu, nv, _ptr(knots_u),
                                      _ptr(knots_v), _stream(stream)), "nurbs_evaluate_random")
    return out


# ----------------------------------------------------------------------------- pools
def pool_check(rc: int, what: str = ""):
    if rc != OK:
        msg = lib().nurbs_pool_last_error().decode(errors="replace")
        raise NurbsError(rc, f"{what}: {msg or lib().nurbs_status_string(rc).decode()}")


class Batch:
    """CSR description of a batch: surface ids[k] owns queries [offsets[k], offsets[k+1])."""

    def __init__(self, ids, offsets):
        self.ids = np.ascontiguousarray(ids, np.int32)
        self.offsets = np.ascontiguousarray(offsets, np.int64)
        assert len(self.offsets) == len(self.ids) + 1

    @property
    def n(self):
        return int(self.offsets[-1] - self.offsets[0]) if len(self.ids) else 0


class Graph:
    def __init__(self, h, keep, pool):
        self.h = h
        self._keep = keep  # device buffers the captured graph reads and writes
        self._pool = pool  # the pool outlives its graphs

    def launch(self, stream=None):
        pool_check(lib().nurbs_graph_launch(self.h, _stream(stream)), "nurbs_graph_launch")

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().nurbs_graph_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Pool:
    """Many surfaces in one device arena under a memory budget (batched workloads, serving)."""

    def __init__(self, budget_bytes: int, max_surfaces: int = 1 << 16):
        h = C.c_void_p()
        pool_check(lib().nurbs_pool_create(int(budget_bytes), int(max_surfaces), C.byref(h)), "nurbs_pool_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().nurbs_pool_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, surfs, stream=None):
        keep, descs = [], (SurfaceDesc * len(surfs))()
        for k, sf in enumerate(surfs):
            arrs = [np.ascontiguousarray(sf[key], np.float64).reshape(-1) for key in ("knots_u", "knots_v", "cps", "weights")]
            keep.append(arrs)
            descs[k] = SurfaceDesc(int(sf["p"]), int(sf["q"]), int(sf["nu"]), int(sf["nv"]),
                                   *(a.ctypes.data for a in arrs))
        ids = np.zeros(len(surfs), np.int32)
        pool_check(lib().nurbs_pool_add(self.h, len(surfs), descs, _stream(stream), ids.ctypes.data), "nurbs_pool_add")
        return ids

    def remove(self, sid: int, stream=None):
        pool_check(lib().nurbs_pool_remove(self.h, int(sid), _stream(stream)), "nurbs_pool_remove")

    def info(self) -> PoolInfo:
        i = PoolInfo()
        pool_check(lib().nurbs_pool_info(self.h, C.byref(i)), "nurbs_pool_info")
        return i

    def set_config(self, tile_queries: int, ctas_per_sm: int):
        pool_check(lib().nurbs_pool_set_config(self.h, tile_queries, ctas_per_sm), "nurbs_pool_set_config")

    def _outs(self, n, dev, out):
        if out is not None:
            return out
        torch = _torch()
        return (torch.empty((n, 2), dtype=torch.float64, device=dev), torch.empty(n, dtype=torch.int32, device=dev),
                torch.empty(n, dtype=torch.float64, device=dev))

    def invert(self, batch: Batch, P, precision: int = PREC_MIXED, stream=None, out=None):
        P = P.contiguous()
        uv, st, res = self._outs(P.shape[0], P.device, out)
        pool_check(lib().nurbs_pool_invert(self.h, len(batch.ids), batch.ids.ctypes.data, batch.offsets.ctypes.data,
                                           _ptr(P), _ptr(uv), _ptr(st), _ptr(res), precision, _stream(stream)),
                   "nurbs_pool_invert")
        return uv, st, res

    def eval(self, batch: Batch, uv, mask: int = S, stream=None):
        torch = _torch()
        uv = uv.contiguous()
        n = uv.shape[0]
        nb = bin(mask & 63).count("1")
        out = torch.empty((3 * nb, n), dtype=torch.float64, device=uv.device)
        pool_check(lib().nurbs_pool_eval(self.h, len(batch.ids), batch.ids.ctypes.data, batch.offsets.ctypes.data,
                                         _ptr(uv), n, mask, _ptr(out), _stream(stream)), "nurbs_pool_eval")
        return out

    def autotune(self, batch: Batch, P, out, precision: int = PREC_MIXED, max_queries: int = 0,
                 cache_path: Optional[str] = None, stream=None):
        uv, st, res = out
        bt, bc, ms = C.c_int(), C.c_int(), C.c_float()
        pool_check(lib().nurbs_pool_autotune(self.h, len(batch.ids), batch.ids.ctypes.data, batch.offsets.ctypes.data,
                                             _ptr(P), _ptr(uv), _ptr(st), _ptr(res), precision, int(max_queries),
                                             cache_path.encode() if cache_path else None, _stream(stream),
                                             C.byref(bt), C.byref(bc), C.byref(ms)), "nurbs_pool_autotune")
        return bt.value, bc.value, ms.value

    def graph(self, batch: Batch, P, out, precision: int = PREC_MIXED) -> Graph:
        uv, st, res = out
        h = C.c_void_p()
        pool_check(lib().nurbs_pool_graph_create(self.h, len(batch.ids), batch.ids.ctypes.data, batch.offsets.ctypes.data,
                                                 _ptr(P), _ptr(uv), _ptr(st), _ptr(res), precision, C.byref(h)),
                   "nurbs_pool_graph_create")
        return Graph(h, (P, uv, st, res), self)


def surface_bytes(surf: dict) -> int:
    """Device bytes one surface takes in a pool."""
    b = C.c_int64()
    ku = np.ascontiguousarray(surf["knots_u"], np.float64)
    kv = np.ascontiguousarray(surf["knots_v"], np.float64)
    pool_check(lib().nurbs_pool_surface_bytes(int(surf["p"]), int(surf["q"]), int(surf["nu"]), int(surf["nv"]),
                                              ku.ctypes.data, kv.ctypes.data, C.byref(b)), "nurbs_pool_surface_bytes")
    return b.value


# ---------------------------------------------------------------------------- serving
class ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_int), ("max_batch_queries", C.c_int64), ("max_batch_requests", C.c_int),
                ("precision", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("batches", C.c_int64), ("batch_queries", C.c_int64), ("in_flight", C.c_int),
                ("gpu_ms", C.c_double), ("dispatch_us", C.c_double), ("retire_us", C.c_double)]


class Server:
    """Continuous-batching inversion service over a pool (threads live in the library)."""

    def __init__(self, pool: Pool, slots: int = 4, max_batch_queries: int = 1 << 16, max_batch_requests: int = 1024,
                 precision: int = PREC_MIXED):
        self.pool = pool
        cfg = ServerConfig(slots, max_batch_queries, max_batch_requests, precision)
        h = C.c_void_p()
        check(lib().nurbs_server_create(pool.h, C.byref(cfg), C.byref(h)), "nurbs_server_create")
        self.h = h
        self._keep = {}

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().nurbs_server_destroy(self.h)
            self.h = C.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit_invert(self, sid: int, P: np.ndarray):
        """Returns (ticket, (uv, status, residual, latency)) host arrays filled on completion."""
        P = np.ascontiguousarray(P, np.float64).reshape(-1, 3)
        n = P.shape[0]
        uv, st, res, lat = np.empty((n, 2)), np.empty(n, np.int32), np.empty(n), np.zeros(1)
        t = C.c_uint64()
        check(lib().nurbs_server_submit_invert(self.h, int(sid), P.ctypes.data, n, uv.ctypes.data, st.ctypes.data,
                                               res.ctypes.data, lat.ctypes.data, C.byref(t)), "submit_invert")
        self._keep[t.value] = (P, uv, st, res, lat)
        return t.value, (uv, st, res, lat)

    def submit_upload(self, surf: dict):
        arrs = [np.ascontiguousarray(surf[k], np.float64).reshape(-1) for k in ("knots_u", "knots_v", "cps", "weights")]
        d = SurfaceDesc(int(surf["p"]), int(surf["q"]), int(surf["nu"]), int(surf["nv"]), *(a.ctypes.data for a in arrs))
        sid, lat = np.full(1, -1, np.int32), np.zeros(1)
        t = C.c_uint64()
        check(lib().nurbs_server_submit_upload(self.h, C.byref(d), sid.ctypes.data, lat.ctypes.data, C.byref(t)),
              "submit_upload")
        self._keep[t.value] = (arrs, d, sid, lat)
        return t.value, sid

    def wait(self, ticket: int, timeout_ms: int = 10000) -> int:
        r = C.c_int()
        rc = lib().nurbs_server_wait(self.h, C.c_uint64(ticket), timeout_ms, C.byref(r))
        if rc == OK:
            self._keep.pop(ticket, None)
            return r.value
        return rc

    def drain(self, timeout_ms: int = 30000) -> int:
        return lib().nurbs_server_drain(self.h, timeout_ms)

    def pause(self, paused: bool):
        check(lib().nurbs_server_pause(self.h, 1 if paused else 0), "pause")

    def stats(self) -> ServerStats:
        s = ServerStats()
        check(lib().nurbs_server_stats(self.h, C.byref(s)), "stats")
        return s

    def replay(self, arrival_us, kind, surf, qoff, P, uploads=(), upload_index=None, timeout_ms=120000):
        """Native replay of a request trace; returns (uv, status, residual, latency_us, results, upload_ids)."""
        nreq = len(arrival_us)
        arrival_us = np.ascontiguousarray(arrival_us, np.float64)
        kind = np.ascontiguousarray(kind, np.int32)
        surf = np.ascontiguousarray(surf, np.int32)
        qoff = np.ascontiguousarray(qoff, np.int64)
        P = np.ascontiguousarray(P, np.float64).reshape(-1, 3)
        n = P.shape[0]
        uv, st, res = np.empty((n, 2)), np.empty(n, np.int32), np.empty(n)
        lat, results = np.zeros(nreq), np.zeros(nreq, np.int32)
        keep = []
        descs = (SurfaceDesc * max(1, len(uploads)))()
        for k, sf in enumerate(uploads):
            arrs = [np.ascontiguousarray(sf[key], np.float64).reshape(-1) for key in ("knots_u", "knots_v", "cps", "weights")]
            keep.append(arrs)
            descs[k] = SurfaceDesc(int(sf["p"]), int(sf["q"]), int(sf["nu"]), int(sf["nv"]), *(a.ctypes.data for a in arrs))
        uidx = np.ascontiguousarray(upload_index if upload_index is not None else np.zeros(nreq), np.int32)
        uids = np.full(max(1, len(uploads)), -1, np.int32)
        rc = lib().nurbs_server_replay(self.h, nreq, arrival_us.ctypes.data, kind.ctypes.data, surf.ctypes.data,
                                       qoff.ctypes.data, P.ctypes.data, uv.ctypes.data, st.ctypes.data, res.ctypes.data,
                                       C.cast(descs, C.c_void_p), uidx.ctypes.data, uids.ctypes.data, lat.ctypes.data,
                                       results.ctypes.data, timeout_ms)
        check(rc, "nurbs_server_replay")
        return uv, st, res, lat, results, uids
