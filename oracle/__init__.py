"""CPU oracle — test infrastructure only.

ctypes bindings for ``liboracle.so`` (the plain-C restatement of the reference's FP64
path, ``nurbs_oracle.c``) and, where it was built, ``_ref/libnurbs_ref.so`` (the
reference's own functions compiled for the host; see ``ref_shim.cu``).  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TREE_NODES = 65
CONE_STRIDE = 20    # floats per node of the FP32 cone records (orc_build_cones)
UPTS = 81           # lattice surface points per node (distance bounds, projection seeds)

S, SU, SV, SUU, SUV, SVV = 1, 2, 4, 8, 16, 32
FOUND_UNIQUE, FOUND_AMBIGUOUS, NO_CANDIDATE, NOT_CONVERGED = 0, 1, 2, 3
# Inversion: iteration cap per trajectory (the CUDA library's FP64 schedule has the same cap),
# and the perturbations of the stability check: K points whose coordinates (relative to the
# control net's centre) are scaled by (1 +- 2^-22) or (1 +- 2^-20), two and eight units of FP32
# rounding.
MAX_ITER = 40
PERTURB_K = 8
PERTURB_EPS = 2.0 ** -22

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_bp = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")


class _Surf(C.Structure):
    _fields_ = [("degree_u", C.c_int), ("degree_v", C.c_int), ("cp_u", C.c_int), ("cp_v", C.c_int),
                ("knots_u", C.c_void_p), ("knots_v", C.c_void_p), ("cps", C.c_void_p), ("weights", C.c_void_p)]


def build(force: bool = False) -> str:
    """Compile liboracle.so in place (gcc, no GPU needed)."""
    so = os.path.join(HERE, "liboracle.so")
    if force or not os.path.exists(so) or os.path.getmtime(so) < max(
            os.path.getmtime(os.path.join(HERE, f)) for f in ("nurbs_oracle.c", "nurbs_oracle.h")):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return so


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        L.orc_matrix_n_size.restype = C.c_int64
        L.orc_matrix_n_size.argtypes = [C.POINTER(_Surf)]
        L.orc_matrix_n.restype = C.c_int
        L.orc_matrix_n.argtypes = [C.POINTER(_Surf), _dp]
        L.orc_eval.restype = None
        L.orc_eval.argtypes = [C.POINTER(_Surf), _dp, _dp, C.c_int64, C.c_uint, _dp, C.c_int]
        L.orc_build_tree.restype = None
        L.orc_build_tree.argtypes = [C.POINTER(_Surf), _dp, _dp, _bp, _bp]
        L.orc_candidates.restype = C.c_int
        L.orc_candidates.argtypes = [_dp, _bp, _dp, _ip]
        L.orc_invert.restype = None
        L.orc_invert.argtypes = [C.POINTER(_Surf), _dp, _dp, _bp, _dp, C.c_int64, C.c_int, _dp, _ip, _dp,
                                 C.c_void_p, C.c_int]
        L.orc_invert_perturbed.restype = None
        L.orc_invert_perturbed.argtypes = [C.POINTER(_Surf), _dp, _dp, _bp, _dp, C.c_int64, C.c_int, C.c_int,
                                           C.c_double, _dp, _ip, _dp, C.c_int]
        L.orc_invert_fp32_explore.restype = None
        L.orc_invert_fp32_explore.argtypes = [C.POINTER(_Surf), _dp, _dp, _bp, _dp, C.c_int64, C.c_int, C.c_int,
                                              C.c_double, _dp, _ip, _dp, C.c_int]
        L.orc_pcurve.restype = None
        L.orc_pcurve.argtypes = [C.POINTER(_Surf), _dp, _dp, _bp, _dp, C.c_int64, C.c_int, _dp, _ip, _dp, _ip,
                                 C.c_int]
        _fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
        L.orc_build_cones.restype = None
        L.orc_build_cones.argtypes = [C.POINTER(_Surf), _dp, _dp, _bp, _dp, _fp, _fp]
        L.orc_project_cull.restype = C.c_int
        L.orc_project_cull.argtypes = [_dp, _bp, _fp, _fp, _dp, _dp, _ip]
        L.orc_project.restype = None
        L.orc_project.argtypes = [C.POINTER(_Surf), _dp, _dp, _bp, _fp, _dp, C.c_int64, C.c_int, _dp, _ip, _dp,
                                  C.c_void_p, C.c_int]
        L.orc_project_perturbed.restype = None
        L.orc_project_perturbed.argtypes = [C.POINTER(_Surf), _dp, _dp, _bp, _fp, _dp, C.c_int64, C.c_int, C.c_int,
                                            C.c_double, _dp, _ip, _dp, C.c_int]
        L.orc_invert_quadtree.restype = None
        L.orc_invert_quadtree.argtypes = [C.POINTER(_Surf), _dp, _dp, C.c_int64, C.c_double, C.c_int, _dp, _ip, _dp,
                                          C.c_void_p, C.c_int]
        L.orc_qt_hull_check.restype = C.c_int
        L.orc_qt_hull_check.argtypes = [C.POINTER(_Surf), _dp, _dp, C.c_double]
        L.orc_qt_split_type.restype = C.c_int
        L.orc_qt_split_type.argtypes = [C.POINTER(_Surf), _dp, _dp, C.c_double, C.c_int]
        L.orc_ders3.restype = None
        L.orc_ders3.argtypes = [C.POINTER(_Surf), _dp, C.c_double, C.c_double, _dp]
        L.orc_normals.restype = None
        L.orc_normals.argtypes = [C.POINTER(_Surf), _dp, C.c_double, C.c_double, _dp]
        L.orc_eval_normal.restype = None
        L.orc_eval_normal.argtypes = [C.POINTER(_Surf), _dp, _dp, C.c_int64, C.c_uint, _dp, C.c_int]
        L.orc_gauss_newton_shipped.restype = C.c_int
        L.orc_gauss_newton_shipped.argtypes = [C.POINTER(_Surf), _dp, _dp, _dp, C.c_double, _dp]
        L.orc_find_span.restype = C.c_int
        L.orc_find_span.argtypes = [C.c_int, C.c_int, _dp, C.c_double]
        L.orc_cube.restype = C.c_double
        L.orc_cube.argtypes = [C.c_double]
        L.orc_point_r.restype = None
        L.orc_point_r.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_double, _dp]
    return _lib


class OracleSurface:
    """Holds contiguous arrays for one surface and the oracle's span matrices / tree."""

    def __init__(self, surf):
        self.p, self.q = int(surf["p"]), int(surf["q"])
        self.nu, self.nv = int(surf["nu"]), int(surf["nv"])
        self.ku = np.ascontiguousarray(surf["knots_u"], dtype=np.float64)
        self.kv = np.ascontiguousarray(surf["knots_v"], dtype=np.float64)
        self.cps = np.ascontiguousarray(surf["cps"], dtype=np.float64).reshape(-1, 3)
        self.w = np.ascontiguousarray(surf["weights"], dtype=np.float64).reshape(-1)
        self._s = _Surf(self.p, self.q, self.nu, self.nv, self.ku.ctypes.data, self.kv.ctypes.data,
                        self.cps.ctypes.data, self.w.ctypes.data)
        self._M = None
        self._tree = None
        self._cones = None

    @property
    def matrix_n(self) -> np.ndarray:
        if self._M is None:
            n = lib().orc_matrix_n_size(C.byref(self._s))
            M = np.zeros(n, dtype=np.float64)
            rc = lib().orc_matrix_n(C.byref(self._s), M)
            if rc < 0:
                raise ValueError("oracle: unsupported surface")
            self._M = M
        return self._M

    def eval(self, uv: np.ndarray, mask: int, threads: int = 0) -> np.ndarray:
        uv = np.ascontiguousarray(uv, dtype=np.float64).reshape(-1, 2)
        n = uv.shape[0]
        nb = bin(mask & 1023).count("1")
        out = np.empty(3 * nb * n, dtype=np.float64)
        lib().orc_eval(C.byref(self._s), self.matrix_n, uv, n, mask, out, threads)
        return out.reshape(3 * nb, n)

    def eval_normal(self, uv: np.ndarray, mask: int, threads: int = 0) -> np.ndarray:
        uv = np.ascontiguousarray(uv, dtype=np.float64).reshape(-1, 2)
        n = uv.shape[0]
        nb = bin(mask & 63).count("1")
        out = np.empty(3 * nb * n, dtype=np.float64)
        lib().orc_eval_normal(C.byref(self._s), self.matrix_n, uv, n, mask, out, threads)
        return out.reshape(3 * nb, n)

    def tree(self):
        if self._tree is None:
            t = np.zeros(TREE_NODES * 10, dtype=np.float64)
            d = np.zeros(TREE_NODES, dtype=np.uint8)
            b = np.zeros(TREE_NODES, dtype=np.uint8)
            lib().orc_build_tree(C.byref(self._s), self.matrix_n, t, d, b)
            self._tree = (t.reshape(TREE_NODES, 10), d, b)
        return self._tree

    def candidates(self, P: np.ndarray):
        t, _, b = self.tree()
        tf = np.ascontiguousarray(t.reshape(-1))
        P = np.ascontiguousarray(P, dtype=np.float64).reshape(-1, 3)
        out = []
        lst = np.zeros(TREE_NODES, dtype=np.int32)
        for k in range(P.shape[0]):
            n = lib().orc_candidates(tf, b, np.ascontiguousarray(P[k]), lst)
            out.append(lst[:n].copy())
        return out

    def invert(self, P: np.ndarray, max_iter: int = MAX_ITER, threads: int = 0):
        t, _, b = self.tree()
        P = np.ascontiguousarray(P, dtype=np.float64).reshape(-1, 3)
        n = P.shape[0]
        uv = np.empty(2 * n, dtype=np.float64)
        st = np.empty(n, dtype=np.int32)
        res = np.empty(n, dtype=np.float64)
        it = np.empty(n, dtype=np.int32)
        lib().orc_invert(C.byref(self._s), self.matrix_n, np.ascontiguousarray(t.reshape(-1)), b, P, n, max_iter,
                         uv, st, res, it.ctypes.data, threads)
        return uv.reshape(n, 2), st, res, it

    def origin(self) -> np.ndarray:
        """Centre of the control net's bounding box (the FP32 arithmetic's origin)."""
        return 0.5 * (self.cps.min(0) + self.cps.max(0))

    def cones(self):
        """Normal boxes (65, 6), FP32 cone records (65, CONE_STRIDE) and distance-bound points
        (65, UPTS, 3) of the built nodes (orc_build_cones)."""
        if self._cones is None:
            t, _, b = self.tree()
            nb = np.zeros(TREE_NODES * 6, dtype=np.float64)
            cr = np.zeros(TREE_NODES * CONE_STRIDE, dtype=np.float32)
            up = np.zeros(TREE_NODES * UPTS * 3, dtype=np.float32)
            lib().orc_build_cones(C.byref(self._s), self.matrix_n, np.ascontiguousarray(t.reshape(-1)), b, nb, cr, up)
            self._cones = (nb.reshape(TREE_NODES, 6), cr.reshape(TREE_NODES, CONE_STRIDE), up.reshape(TREE_NODES, UPTS, 3))
        return self._cones

    def _cone_arg(self):
        _, cr, up = self.cones()
        return np.ascontiguousarray(np.concatenate([cr.reshape(-1), up.reshape(-1)]))

    def project_candidates(self, P: np.ndarray):
        """Per point: the projection's candidates, 128 * node + the seed's lattice index."""
        t, _, b = self.tree()
        _, cr, up = self.cones()
        cr = np.ascontiguousarray(cr.reshape(-1))
        up = np.ascontiguousarray(up.reshape(-1))
        tf = np.ascontiguousarray(t.reshape(-1))
        org = np.ascontiguousarray(self.origin())
        P = np.ascontiguousarray(P, dtype=np.float64).reshape(-1, 3)
        lst = np.zeros(TREE_NODES, dtype=np.int32)
        out = []
        for k in range(P.shape[0]):
            n = lib().orc_project_cull(tf, b, cr, up, np.ascontiguousarray(P[k]), org, lst)
            out.append(lst[:n].copy())
        return out

    def project(self, P: np.ndarray, max_iter: int = MAX_ITER, threads: int = 0):
        """Closest point over the closed domain (orc_project): uv (n,2), status, residual, iters."""
        t, _, b = self.tree()
        cr = self._cone_arg()
        P = np.ascontiguousarray(P, dtype=np.float64).reshape(-1, 3)
        n = P.shape[0]
        uv = np.empty(2 * n, dtype=np.float64)
        st = np.empty(n, dtype=np.int32)
        res = np.empty(n, dtype=np.float64)
        it = np.empty(n, dtype=np.int32)
        lib().orc_project(C.byref(self._s), self.matrix_n, np.ascontiguousarray(t.reshape(-1)), b, cr, P, n,
                          max_iter, uv, st, res, it.ctypes.data, threads)
        return uv.reshape(n, 2), st, res, it

    def invert_perturbed(self, P: np.ndarray, K: int = PERTURB_K, eps: float = PERTURB_EPS, max_iter: int = MAX_ITER,
                         threads: int = 0, project: bool = False):
        """Answers for K perturbations of P at FP32 resolution, carried back to P (see
        orc_invert_perturbed; project: of the projection): uv (K, n, 2), found (K, n) bool,
        residual (K, n)."""
        t, _, b = self.tree()
        P = np.ascontiguousarray(P, dtype=np.float64).reshape(-1, 3)
        n = P.shape[0]
        uv = np.empty(2 * K * n, dtype=np.float64)
        found = np.empty(K * n, dtype=np.int32)
        res = np.empty(K * n, dtype=np.float64)
        tf = np.ascontiguousarray(t.reshape(-1))
        if project:
            lib().orc_project_perturbed(C.byref(self._s), self.matrix_n, tf, b,
                                        self._cone_arg(), P, n, max_iter, K, eps, uv,
                                        found, res, threads)
        else:
            lib().orc_invert_perturbed(C.byref(self._s), self.matrix_n, tf, b, P, n, max_iter, K, eps, uv, found,
                                       res, threads)
        return uv.reshape(K, n, 2), found.reshape(K, n).astype(bool), res.reshape(K, n)

    def invert_fp32_explore(self, P: np.ndarray, perturbation: int = -1, eps: float = PERTURB_EPS,
                            max_iter: int = MAX_ITER, threads: int = 0):
        """The inversion with its exploration in FP32 arithmetic (orc_invert_fp32_explore), of the
        points or of their perturbation `perturbation` (>= 0): uv (n, 2), found (n,) bool,
        residual (n,), all for the true points."""
        t, _, b = self.tree()
        P = np.ascontiguousarray(P, dtype=np.float64).reshape(-1, 3)
        n = P.shape[0]
        uv = np.empty(2 * n, dtype=np.float64)
        found = np.empty(n, dtype=np.int32)
        res = np.empty(n, dtype=np.float64)
        lib().orc_invert_fp32_explore(C.byref(self._s), self.matrix_n, np.ascontiguousarray(t.reshape(-1)), b, P, n,
                                      max_iter, perturbation, eps, uv, found, res, threads)
        return uv.reshape(n, 2), found.astype(bool), res

    def stability_set(self, P: np.ndarray, threads: int = 0, project: bool = False):
        """The oracle's answers at FP32 resolution, for parity.classify_inversion: the answers
        for the PERTURB_K perturbed points (FP64), and those of the FP32 exploration of the points
        and of the same perturbed points, all carried to the true points; stacked (2K+1, n, ...).
        project: of the projection, whose GPU arithmetic is FP64: the K perturbed answers only."""
        pu, pf, pr = self.invert_perturbed(P, threads=threads, project=project)
        if project:
            return pu, pf, pr
        us, fs, rs = [pu], [pf], [pr]
        for k in range(-1, PERTURB_K):
            fu, ff, fr = self.invert_fp32_explore(P, perturbation=k, threads=threads)
            us.append(fu[None])
            fs.append(ff[None])
            rs.append(fr[None])
        return np.concatenate(us), np.concatenate(fs), np.concatenate(rs)

    def pcurve(self, Cs: np.ndarray, max_iter: int = MAX_ITER, threads: int = 0):
        """p-curve of ordered curve samples (orc_pcurve): uv (n,2), status, residual, flags."""
        t, _, b = self.tree()
        Cs = np.ascontiguousarray(Cs, dtype=np.float64).reshape(-1, 3)
        n = Cs.shape[0]
        uv = np.empty(2 * n, dtype=np.float64)
        st = np.empty(n, dtype=np.int32)
        res = np.empty(n, dtype=np.float64)
        fl = np.empty(n, dtype=np.int32)
        lib().orc_pcurve(C.byref(self._s), self.matrix_n, np.ascontiguousarray(t.reshape(-1)), b, Cs, n, max_iter,
                         uv, st, res, fl, threads)
        return uv.reshape(n, 2), st, res, fl

    def invert_quadtree(self, P: np.ndarray, max_edge: float, max_iter: int = MAX_ITER, threads: int = 0):
        """Adaptive quadtree inversion (orc_invert_quadtree): uv (n,2), status, residual, layers."""
        P = np.ascontiguousarray(P, dtype=np.float64).reshape(-1, 3)
        n = P.shape[0]
        uv = np.empty(2 * n, dtype=np.float64)
        st = np.empty(n, dtype=np.int32)
        res = np.empty(n, dtype=np.float64)
        ly = np.empty(n, dtype=np.int32)
        lib().orc_invert_quadtree(C.byref(self._s), self.matrix_n, P, n, max_edge, max_iter, uv, st, res,
                                  ly.ctypes.data, threads)
        return uv.reshape(n, 2), st, res, ly

    def qt_hull_check(self, node4, P, max_edge):
        return int(lib().orc_qt_hull_check(C.byref(self._s), np.ascontiguousarray(node4, np.float64),
                                           np.ascontiguousarray(P, np.float64), max_edge))

    def qt_split_type(self, node4, max_edge, as_reference=False):
        return int(lib().orc_qt_split_type(C.byref(self._s), self.matrix_n, np.ascontiguousarray(node4, np.float64),
                                           max_edge, 1 if as_reference else 0))

    def ders3(self, u, v):
        """S..Svvv (10, 3) and N, Nu, Nv, Nuu, Nuv, Nvv (6, 3) at one parameter pair."""
        d = np.zeros(30)
        nrm = np.zeros(18)
        lib().orc_ders3(C.byref(self._s), self.matrix_n, float(u), float(v), d)
        lib().orc_normals(C.byref(self._s), self.matrix_n, float(u), float(v), nrm)
        return d.reshape(10, 3), nrm.reshape(6, 3)

    def gauss_newton_shipped(self, seed, P, max_edge):
        uv = np.zeros(2)
        ok = lib().orc_gauss_newton_shipped(C.byref(self._s), self.matrix_n, np.asarray(seed, np.float64),
                                            np.asarray(P, np.float64), max_edge, uv)
        return bool(ok), uv


# ------------------------------------------------------------------ reference shim
_ref = None


def ref_lib():
    """The reference's own functions compiled for the host (only where oracle/_ref was built)."""
    global _ref
    if _ref is None:
        so = os.path.join(HERE, "_ref", "libnurbs_ref.so")
        if not os.path.exists(so):
            return None
        R = C.CDLL(so)
        R.ref_matrix_n.restype = C.c_int
        R.ref_matrix_n.argtypes = [C.c_int] * 4 + [_dp, _dp, _dp, _dp, _dp]
        R.ref_eval.restype = None
        R.ref_eval.argtypes = [C.c_int] * 4 + [_dp, _dp, _dp, _dp, C.c_longlong, C.c_uint, _dp]
        R.ref_build_tree.restype = None
        R.ref_build_tree.argtypes = [C.c_int] * 4 + [_dp, _dp, _dp, _dp, _bp, _bp]
        R.ref_box_check.restype = C.c_int
        R.ref_box_check.argtypes = [_dp, _dp]
        R.ref_gauss_newton.restype = C.c_int
        R.ref_gauss_newton.argtypes = [C.c_int] * 4 + [_dp, _dp, _dp, _dp, _dp, C.c_double, _dp]
        R.ref_find_span.restype = C.c_int
        R.ref_find_span.argtypes = [C.c_int, C.c_int, _dp, C.c_double]
        R.ref_ders3.restype = None
        R.ref_ders3.argtypes = [C.c_int] * 4 + [_dp, _dp, _dp, C.c_double, C.c_double, _dp]
        R.ref_qt_box_check.restype = C.c_int
        R.ref_qt_box_check.argtypes = [C.c_int] * 4 + [_dp, _dp, _dp, _dp, _dp, C.c_double]
        R.ref_qt_split_type.restype = C.c_int
        R.ref_qt_split_type.argtypes = [C.c_int] * 4 + [_dp, _dp, _dp, _dp, C.c_double]
        _ref = R
    return _ref


class RefSurface:
    """Same interface as OracleSurface, backed by the reference's own compiled functions."""

    def __init__(self, surf):
        self.o = OracleSurface(surf)
        self.R = ref_lib()
        if self.R is None:
            raise RuntimeError("oracle/_ref not built")
        self._M = None
        self._tree = None

    def _dims(self):
        o = self.o
        return (o.p, o.q, o.nu, o.nv)

    @property
    def matrix_n(self):
        if self._M is None:
            o = self.o
            M = np.zeros(lib().orc_matrix_n_size(C.byref(o._s)), dtype=np.float64)
            self.R.ref_matrix_n(*self._dims(), o.ku, o.kv, np.ascontiguousarray(o.cps.reshape(-1)), o.w, M)
            self._M = M
        return self._M

    def eval(self, uv, mask):
        uv = np.ascontiguousarray(uv, dtype=np.float64).reshape(-1, 2)
        n = uv.shape[0]
        nb = bin(mask & 63).count("1")
        out = np.empty(3 * nb * n, dtype=np.float64)
        self.R.ref_eval(*self._dims(), self.o.ku, self.o.kv, self.matrix_n, uv, n, mask, out)
        return out.reshape(3 * nb, n)

    def tree(self):
        if self._tree is None:
            t = np.zeros(TREE_NODES * 10, dtype=np.float64)
            d = np.zeros(TREE_NODES, dtype=np.uint8)
            b = np.zeros(TREE_NODES, dtype=np.uint8)
            self.R.ref_build_tree(*self._dims(), self.o.ku, self.o.kv, self.matrix_n, t, d, b)
            self._tree = (t.reshape(TREE_NODES, 10), d, b)
        return self._tree

    def candidates(self, P):
        t, _, b = self.tree()
        P = np.ascontiguousarray(P, dtype=np.float64).reshape(-1, 3)
        out = []
        for k in range(P.shape[0]):
            pk = np.ascontiguousarray(P[k])
            out.append(np.array([i for i in range(TREE_NODES)
                                 if b[i] and self.R.ref_box_check(np.ascontiguousarray(t[i]), pk)], dtype=np.int32))
        return out

    def ders3(self, u, v):
        """The reference's new-style derivatives (14, 3): S..Svvv, N, Nuu, Nuv, Nvv."""
        out = np.zeros(42)
        self.R.ref_ders3(*self._dims(), self.o.ku, self.o.kv, self.matrix_n, float(u), float(v), out)
        return out.reshape(14, 3)

    def qt_box_check(self, node4, P, max_edge):
        return int(self.R.ref_qt_box_check(*self._dims(), self.o.ku, self.o.kv,
                                           np.ascontiguousarray(self.o.cps.reshape(-1)),
                                           np.ascontiguousarray(node4, np.float64),
                                           np.ascontiguousarray(P, np.float64), max_edge))

    def qt_split_type(self, node4, max_edge):
        return int(self.R.ref_qt_split_type(*self._dims(), self.o.ku, self.o.kv, self.matrix_n,
                                            np.ascontiguousarray(node4, np.float64), max_edge))

    def gauss_newton_shipped(self, node_uv4, P, max_edge):
        uv = np.zeros(2)
        ok = self.R.ref_gauss_newton(*self._dims(), self.o.ku, self.o.kv, self.matrix_n,
                                     np.asarray(node_uv4, np.float64), np.asarray(P, np.float64), max_edge, uv)
        return bool(ok), uv
