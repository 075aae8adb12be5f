"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run in a checkout where the reference tree is available and oracle/_ref has been built
(``make -C oracle ref REF_DIR=<reference>``):

    python tests/golden/make_golden.py --ref-dir /path/to/GPU-NURBS

For each of the reference's sample models (model/*.nu) and for the small synthetic surface it
records, computed by the reference's own FP64 functions compiled for the host:
  * the parsed surface (degree, net, knots, control points, weights),
  * MatrixN (GetMatrixN, bit patterns),
  * S, Su, Sv, Suu, Suv, Svv at 256 parameter pairs including the domain corners,
  * the 2-level tree (boxes, Divided, built) and candidate lists of 128 query points,
  * the shipped GaussNewton result from a few seeds (max_edge 0.01, 1e-4),
and the two known-answer points hard-coded in src/kernel/kernel.cu:452-454.
"""
from __future__ import annotations

import argparse
import glob
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def parse_nu_text(text: str) -> dict:
    """Minimal reader of the .nu grammar (tags NU, CP, KNu, KNv, DP), for fixture making only."""
    it = iter([l.split() for l in text.splitlines()])

    def find(tag):
        for toks in it:
            if toks and toks[0] == tag:
                return toks[1:]
        raise ValueError(f"missing tag {tag}")

    p, q = map(int, find("NU")[:2])
    nu, nv = map(int, find("CP")[:2])
    ku = np.array(list(map(float, find("KNu")[: p + nu + 1])))
    kv = np.array(list(map(float, find("KNv")[: q + nv + 1])))
    cps = np.zeros((nu * nv, 3))
    w = np.zeros(nu * nv)
    for k in range(nu * nv):
        x = list(map(float, find("DP")[:4]))
        cps[k] = x[:3]
        w[k] = x[3]
    return dict(p=p, q=q, nu=nu, nv=nv, knots_u=ku, knots_v=kv, cps=cps, weights=w)


def fixture(name: str, surf: dict, rng: np.random.Generator) -> dict:
    import oracle as O
    R = O.RefSurface(surf)
    uv = rng.random((256, 2))
    uv[:6] = [[0, 0], [1, 1], [0, 1], [1, 0], [0.25, 0.25], [0.5, 0.5]]
    ev = R.eval(uv, 63)
    tree, div, built = R.tree()
    S = R.eval(rng.random((128, 2)), 7)
    nrm = np.cross(S[3:6].T, S[6:9].T)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    P = S[0:3].T + rng.normal(0, 0.02, (128, 1)) * nrm
    P[:8] = S[0:3].T[:8]                   # points on the surface
    cands = R.candidates(P)
    cand_counts = np.array([len(c) for c in cands], np.int32)
    cand_flat = np.concatenate(cands).astype(np.int32) if len(cands) else np.zeros(0, np.int32)
    gn = []
    for k in range(16):
        for me in (0.01, 1e-4):
            node = tree[0] if built[0] else np.array([0, 0, 1, 1.0])
            ok, r_uv = R.gauss_newton_shipped(node[:4], P[k], me)
            gn.append([k, me, float(ok), r_uv[0], r_uv[1]])
    return dict(name=name, p=surf["p"], q=surf["q"], nu=surf["nu"], nv=surf["nv"], knots_u=surf["knots_u"],
                knots_v=surf["knots_v"], cps=surf["cps"], weights=surf["weights"], matrix_n=R.matrix_n,
                uv=uv, eval=ev, tree=tree, divided=div, built=built, P=P, cand_counts=cand_counts,
                cand_flat=cand_flat, gn_shipped=np.array(gn))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-dir", default=os.environ.get("REF_DIR", "/root/reference"))
    a = ap.parse_args()
    import oracle as O
    if O.ref_lib() is None:
        sys.exit("oracle/_ref/libnurbs_ref.so is not built: make -C oracle ref REF_DIR=...")
    rng = np.random.default_rng(20240614)
    models = sorted(glob.glob(os.path.join(a.ref_dir, "model", "*.nu")))
    for path in models:
        name = os.path.splitext(os.path.basename(path))[0]
        surf = parse_nu_text(open(path).read())
        np.savez_compressed(os.path.join(HERE, f"model_{name}.npz"), **fixture(name, surf, rng))
        print("wrote", name)
    from importlib import util
    spec = util.spec_from_file_location("synth", os.path.join(ROOT, "gpu-nurbs_gb300", "synth.py"))
    synth = util.module_from_spec(spec)
    spec.loader.exec_module(synth)
    np.savez_compressed(os.path.join(HERE, "synth_small.npz"), **fixture("synth_small", synth.surface_small(), rng))
    print("wrote synth_small")
    # known-answer points of the reference (src/kernel/kernel.cu:452, 454): S(0.25, 0.25)
    kat = {}
    for name in ("center_bk", "test_face2"):
        surf = parse_nu_text(open(os.path.join(a.ref_dir, "model", f"{name}.nu")).read())
        kat[name] = O.RefSurface(surf).eval(np.array([[0.25, 0.25]]), 1).ravel()
    np.savez(os.path.join(HERE, "kat.npz"), **kat,
             center_bk_ref=np.array([0.000000, 0.200049, 0.616000]),
             test_face2_ref=np.array([0.700000, 0.455556, 0.055556]))
    print("wrote kat")


if __name__ == "__main__":
    main()
