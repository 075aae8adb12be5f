"""Generates tests/golden/pin3_*.npz from the reference itself: the projection path's third-order
and normal derivatives, and the first (quadtree) inversion's control-point box checks and split
types, computed by the reference's own FP64 functions compiled for the host (oracle/_ref, built
by ``make -C oracle ref REF_DIR=<reference>``).

    python tests/golden/make_pins.py

For each surface of the existing fixtures (model_*.npz, synth_small.npz) it records
  * ders3: S, Su, Sv, Suu, Suv, Svv, Suuu, Suuv, Suvv, Svvv, N, Nuu, Nuv, Nvv at 64 parameter
    pairs (MatrixSurfaceRd*, the new-style quotient forms, SurfaceNormalDerivative*),
  * box / split: BoundingBoxCheck of 40 nodes x 48 points and getSplitType of the 40 nodes, for
    max_edge 1e-2 and 1e-4.
"""
from __future__ import annotations

import glob
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def nodes_of(rng):
    """Dyadic squares of depth 0..4 (a sample) and halves of depth-2 squares split one way."""
    out = [[0.0, 0.0, 1.0, 1.0]]
    for d in range(1, 5):
        side = 1 << d
        for _ in range(6):
            a, b = rng.integers(0, side, 2)
            out.append([a / side, b / side, (a + 1) / side, (b + 1) / side])
    for _ in range(7):
        a, b = rng.integers(0, 4, 2)
        lu, lv, ru, rv = a / 4, b / 4, (a + 1) / 4, (b + 1) / 4
        out.append([lu, lv, (lu + ru) / 2, rv])
        out.append([lu, lv, ru, (lv + rv) / 2])
    return np.array(out[:40])


def pins(g, rng):
    import oracle as O
    surf = dict(p=int(g["p"]), q=int(g["q"]), nu=int(g["nu"]), nv=int(g["nv"]), knots_u=g["knots_u"],
                knots_v=g["knots_v"], cps=g["cps"], weights=g["weights"])
    R = O.RefSurface(surf)
    uv = rng.random((64, 2))
    uv[:4] = [[0.3, 0.3], [0.5, 0.5], [0.71, 0.13], [0.9, 0.95]]
    ders3 = np.stack([R.ders3(u, v) for u, v in uv])
    nodes = nodes_of(rng)
    E = R.eval(rng.random((48, 2)), 7)
    nrm = np.cross(E[3:6].T, E[6:9].T)
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-300)
    ext = np.ptp(np.asarray(surf["cps"]).reshape(-1, 3), 0).max()
    P = E[0:3].T + nrm * rng.normal(0, 0.01 * ext, (48, 1))
    P[40:] = np.asarray(surf["cps"]).reshape(-1, 3).mean(0) + (rng.random((8, 3)) - 0.5) * 4 * ext
    box = np.zeros((2, len(nodes), len(P)), np.uint8)
    split = np.zeros((2, len(nodes)), np.int8)
    for e, me in enumerate((1e-2, 1e-4)):
        for i, nd in enumerate(nodes):
            split[e, i] = R.qt_split_type(nd, me)
            for j, x in enumerate(P):
                box[e, i, j] = R.qt_box_check(nd, x, me)
    return dict(uv=uv, ders3=ders3, nodes=nodes, P=P, max_edge=np.array([1e-2, 1e-4]), box=box, split=split)


def main():
    import oracle as O
    if O.ref_lib() is None:
        sys.exit("oracle/_ref/libnurbs_ref.so is not built: make -C oracle ref REF_DIR=...")
    rng = np.random.default_rng(20261204)
    for path in sorted(glob.glob(os.path.join(HERE, "model_*.npz")) + [os.path.join(HERE, "synth_small.npz")]):
        g = np.load(path)
        name = os.path.basename(path)[:-4]
        np.savez_compressed(os.path.join(HERE, f"pin3_{name}.npz"), **pins(g, rng))
        print("wrote pin3", name)


if __name__ == "__main__":
    main()
