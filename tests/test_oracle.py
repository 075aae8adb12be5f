"""CPU tests: the C oracle against the golden fixtures made by the reference's own code.

The fixtures (tests/golden/*.npz) were produced by the reference's FP64 functions compiled for
the host (oracle/_ref, see tests/golden/make_golden.py).  These tests pin the oracle: span
matrices, evaluation, tree and candidate lists must agree bit for bit.
"""
import glob
import math
import os
from fractions import Fraction

import numpy as np
import pytest

import oracle as O
from conftest import golden_files, load_golden, GOLDEN
from parity import classify_inversion, eval_errors, stable_mask

MODEL_FILES = [f for f in golden_files() if os.path.basename(f).startswith(("model_", "synth_"))]


def surf_of(g):
    return dict(p=g["p"], q=g["q"], nu=g["nu"], nv=g["nv"], knots_u=g["knots_u"], knots_v=g["knots_v"],
                cps=g["cps"], weights=g["weights"])


@pytest.mark.parametrize("path", MODEL_FILES, ids=lambda p: os.path.basename(p)[:-4])
def test_matrix_n_bit_exact(path):
    g = load_golden(path)
    o = O.OracleSurface(surf_of(g))
    assert np.array_equal(o.matrix_n.view(np.int64), g["matrix_n"].view(np.int64))


@pytest.mark.parametrize("path", MODEL_FILES, ids=lambda p: os.path.basename(p)[:-4])
def test_eval_bit_exact(path):
    g = load_golden(path)
    o = O.OracleSurface(surf_of(g))
    ev = o.eval(g["uv"], 63)
    assert np.array_equal(ev, g["eval"], equal_nan=True)


@pytest.mark.parametrize("path", MODEL_FILES, ids=lambda p: os.path.basename(p)[:-4])
def test_tree_and_candidates_exact(path):
    g = load_golden(path)
    o = O.OracleSurface(surf_of(g))
    tree, div, built = o.tree()
    assert np.array_equal(built, g["built"])
    b = built == 1
    assert np.array_equal(tree[b], g["tree"][b], equal_nan=True)
    assert np.array_equal(div[b], g["divided"][b])
    cands = o.candidates(g["P"])
    counts = np.array([len(c) for c in cands], np.int32)
    assert np.array_equal(counts, g["cand_counts"])
    flat = np.concatenate(cands) if len(cands) else np.zeros(0, np.int32)
    assert np.array_equal(flat, g["cand_flat"])


@pytest.mark.parametrize("path", MODEL_FILES, ids=lambda p: os.path.basename(p)[:-4])
def test_shipped_gauss_newton_exact(path):
    g = load_golden(path)
    o = O.OracleSurface(surf_of(g))
    tree, _, built = o.tree()
    for k, me, ok, u, v in g["gn_shipped"]:
        node = tree[0] if built[0] else np.array([0, 0, 1, 1.0])
        seed = np.array([(node[0] + node[2]) / 2, (node[1] + node[3]) / 2])
        got_ok, uv = o.gauss_newton_shipped(seed, g["P"][int(k)], me)
        assert got_ok == bool(ok)
        if got_ok:
            assert uv[0] == u and uv[1] == v


def test_known_answer_points():
    """S(0.25,0.25) of center_bk / test_face2 as hard-coded in src/kernel/kernel.cu:452-454."""
    kat = np.load(os.path.join(GOLDEN, "kat.npz"))
    for name in ("center_bk", "test_face2"):
        g = load_golden(os.path.join(GOLDEN, f"model_{name}.npz"))
        S = O.OracleSurface(surf_of(g)).eval(np.array([[0.25, 0.25]]), 1).ravel()
        assert np.array_equal(S, kat[name])
        # the reference prints 6 decimals
        assert np.allclose(S, kat[f"{name}_ref"], atol=5e-7)


def test_cube_is_correctly_rounded():
    """The oracle's pow(h,3) is the once-rounded cube; check against exact rationals."""
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.random(3000) * 10 - 5, rng.random(1000) * 1e-3, [0.5, 1.0, 2.0, 3.0, 1.1]])
    for x in xs:
        x = float(x)
        assert O.lib().orc_cube(x) == float(Fraction(x) ** 3)


def test_find_span_semantics():
    """findSpan (src/NURBS/Evaluate.cu:504-533): clamping and repeated interior knots."""
    k = np.array([0, 0, 0, 0.25, 0.25, 0.5, 0.5, 0.75, 0.75, 1, 1, 1], np.float64)
    f = lambda u: O.lib().orc_find_span(2, 9, k, u)
    assert f(-1.0) == 2 and f(0.0) == 2
    assert f(0.25) == 4 and f(0.2499) == 2
    assert f(1.0) == 8 and f(2.0) == 8
    assert f(0.75) == 8


def test_oracle_inversion_small_recovers_truth():
    """On the small bicubic surface the converged GN oracle recovers the generating (u,v)."""
    from gpu_nurbs_gb300 import synth
    surf = synth.surface_small()
    o = O.OracleSurface(surf)
    uv, off = synth.query_params(300, 11, "small")
    E = o.eval(uv, 7)
    P = synth.form_queries(E[0:3].T, E[3:6].T, E[6:9].T, off)
    ruv, st, res, _ = o.invert(P)
    ok = st == O.FOUND_UNIQUE
    assert ok.mean() > 0.95
    assert np.abs(ruv[ok] - uv[ok]).max() < 1e-12
    assert np.allclose(res[ok], np.abs(off[ok]), rtol=1e-6, atol=1e-12)


def test_oracle_high_degree_eval_against_40_digit_values():
    """Pins the high-degree accuracy fixture: the oracle (the reference's FP64 formulation) is
    within its conditioning-limited error of the 40-digit values."""
    z = np.load(os.path.join(GOLDEN, "eval_truth.npz"))
    for d in z["degrees"]:
        tag = f"p{int(d[0])}q{int(d[1])}_"
        sf = {k: z[tag + k] for k in ("knots_u", "knots_v", "cps", "weights")}
        sf.update({k: int(z[tag + k]) for k in ("p", "q", "nu", "nv")})
        errs = eval_errors(O.OracleSurface(sf).eval(z[tag + "uv"], 63), z[tag + "truth"])
        assert max(errs) < 1e-9, (tag, errs)


def _large_sample(n, seed=21):
    from gpu_nurbs_gb300 import synth
    surf = synth.surface_large()
    o = O.OracleSurface(surf)
    uv, off = synth.query_params(n, seed, "large")
    E = o.eval(uv, 7)
    return o, synth.form_queries(E[0:3].T, E[3:6].T, E[6:9].T, off)


def test_oracle_answers_are_local_minima():
    """The oracle's definition (GN update, then Newton steps once the step is below 1e-2) pins
    nearly every query of the 64x64 workload, and every answer is a minimum of the distance:
    the gradient J^T r vanishes to rounding and the Hessian J^T J + r.d2S is positive definite."""
    o, P = _large_sample(2048)
    uv, st, res, _ = o.invert(P)
    found = st <= 1
    assert (st == O.NOT_CONVERGED).mean() < 0.005
    E = o.eval(uv[found], 63)
    S, Su, Sv, Suu, Suv, Svv = (E[3 * b:3 * b + 3].T for b in range(6))
    r = S - P[found]
    g = np.stack([(Su * r).sum(1), (Sv * r).sum(1)], 1)
    scale = np.linalg.norm(r, axis=1) * np.maximum(np.linalg.norm(Su, axis=1), np.linalg.norm(Sv, axis=1))
    assert np.all(np.abs(g).max(1) <= 1e-9 * np.maximum(scale, 1e-300) + 1e-15)
    h00 = (Su * Su).sum(1) + (r * Suu).sum(1)
    h01 = (Su * Sv).sum(1) + (r * Suv).sum(1)
    h11 = (Sv * Sv).sum(1) + (r * Svv).sum(1)
    assert np.all(h00 > 0) and np.all(h00 * h11 - h01 * h01 > 0)
    assert np.allclose(res[found], np.linalg.norm(r, axis=1), rtol=1e-12, atol=1e-15)


def test_oracle_stability_set_on_a_well_conditioned_surface():
    """On the 8x8 surface with 1e-3 offsets the FP64 answer survives every FP32-resolution
    perturbation and the FP32 exploration: no query is UNSTABLE."""
    from gpu_nurbs_gb300 import synth
    surf = synth.surface_small()
    o = O.OracleSurface(surf)
    uv, off = synth.query_params(2000, 12, "small")
    E = o.eval(uv, 7)
    P = synth.form_queries(E[0:3].T, E[3:6].T, E[6:9].T, off)
    ouv, ost, ores, _ = o.invert(P)
    pset = o.stability_set(P)
    assert pset[0].shape == (2 * O.PERTURB_K + 1, len(P), 2)
    uniq = ost == O.FOUND_UNIQUE
    assert np.array_equal(stable_mask(ouv, ost, pset), uniq)
    fu, ff, fr = o.invert_fp32_explore(P)
    assert np.abs(fu[uniq] - ouv[uniq]).max() <= 1e-12


def test_parity_classifier_catches_planted_mistakes():
    """A wrong minimum on a stable query fails; on an UNSTABLE query a result no worse than the
    oracle's farthest answer passes and a farther one fails; a missing answer fails."""
    o, P = _large_sample(3000, seed=22)
    ouv, ost, ores, _ = o.invert(P)
    pset = o.stability_set(P)
    stable = stable_mask(ouv, ost, pset)
    unstable = (ost == O.FOUND_UNIQUE) & ~stable
    assert unstable.sum() >= 1 and unstable.mean() < 0.01
    uv, st, res = ouv.copy(), ost.copy(), ores.copy()
    c = classify_inversion(uv, st, res, ouv, ost, ores, P, perturbed=pset)
    assert c["fail_unique"] == c["fail_unstable"] == 0 and c["unstable"] == unstable.sum()
    i = int(np.nonzero(stable)[0][0])
    uv[i] += 1e-8                       # another point of the same minimum's neighbourhood
    res[i] *= 1 + 1e-9
    st[int(np.nonzero(stable)[0][1])] = O.NOT_CONVERGED
    j = int(np.nonzero(unstable)[0][0])
    worst = np.nanmax(np.where(pset[1][:, j], pset[2][:, j], -np.inf))
    uv[j] = [0.123, 0.456]
    res[j] = max(worst, ores[j]) * 1.01  # farther than every answer the oracle gives
    c = classify_inversion(uv, st, res, ouv, ost, ores, P, perturbed=pset)
    assert c["fail_unique"] == 2 and c["fail_unstable"] == 1
    res[j] = max(worst, ores[j])         # as far as the farthest: passes
    c = classify_inversion(uv, st, res, ouv, ost, ores, P, perturbed=pset)
    assert c["fail_unstable"] == 0


def tube(nu=12, nv=5):
    """A bicubic tube: control rows on a circle whose first and last rows coincide, so the
    surface closes (C0) where u = 0 meets u = 1 and a curve around it crosses that seam."""
    from gpu_nurbs_gb300 import synth
    a = 2 * np.pi * np.arange(nu) / (nu - 1)
    x = np.repeat(np.cos(a), nv)
    y = np.repeat(np.sin(a), nv)
    z = np.tile(np.arange(nv) / (nv - 1), nu)
    return dict(p=3, q=3, nu=nu, nv=nv, knots_u=synth.uniform_knots(3, nu), knots_v=synth.uniform_knots(3, nv),
                cps=np.stack([x, y, z], 1), weights=np.ones(nu * nv))


def test_oracle_pcurve_recovers_a_loop_and_flags_a_jump():
    """The oracle's p-curve: a loop on the 64x64 surface comes back to 1e-12 with no flags; on a
    tube, a curve around it crosses the seam u = 1 -> 0, where the parameter jumps although the
    curve does not: flagged there and nowhere else."""
    from gpu_nurbs_gb300 import synth
    o = O.OracleSurface(synth.surface_large())
    t = np.linspace(0, 1, 801)
    uv = np.stack([0.5 + 0.3 * np.cos(2 * np.pi * t), 0.5 + 0.2 * np.sin(4 * np.pi * t)], 1)
    C = o.eval(uv, 1).T.copy()
    ruv, st, res, fl = o.pcurve(C)
    assert np.all(st == O.FOUND_UNIQUE)
    assert np.abs(ruv - uv).max() <= 1e-12
    assert np.count_nonzero(fl) == 0
    ot = O.OracleSurface(tube())
    u = (0.3 + np.arange(300) / 250.0 + 0.5 / 250) % 1.0
    uvt = np.stack([u, np.full(300, 0.4)], 1)
    Ct = ot.eval(uvt, 1).T.copy()
    ruv, st, res, fl = ot.pcurve(Ct)
    wrap = int(np.nonzero(np.diff(u) < 0)[0][0]) + 1
    assert np.all(st <= O.FOUND_AMBIGUOUS)
    assert fl[wrap] & 1 and np.count_nonzero(fl & 1) == 1
    assert np.abs(ruv - uvt).max() <= 1e-10


def _fd_sample(surf, n, seed):
    rng = np.random.default_rng(seed)
    return np.clip(rng.random((n, 2)), 0.02, 0.98)


@pytest.mark.parametrize("kind", ["large", "quintic", "rational"])
def test_oracle_third_derivatives_and_normals_against_differences(kind):
    """Third derivatives (Suuu, Suuv, Suvv, Svvv) and the normal's derivatives against central
    differences of the orders below them, away from span boundaries; and N = Su x Sv against the
    first derivatives of the reference-order evaluation."""
    from gpu_nurbs_gb300 import synth
    if kind == "large":
        surf = synth.surface_large()
    elif kind == "quintic":
        surf = synth.surface_quintic(n=16)
    else:
        surf = synth.surface_random(synth.Rng(77))
    o = O.OracleSurface(surf)
    ku = np.unique(surf["knots_u"])
    kv = np.unique(surf["knots_v"])
    uv = _fd_sample(surf, 400, 5)
    h = 1e-6
    # keep both sides of every difference inside one span
    du = np.abs(uv[:, :1] - ku[None, :]).min(1)
    dv = np.abs(uv[:, 1:] - kv[None, :]).min(1)
    uv = uv[(du > 10 * h) & (dv > 10 * h)]
    n = len(uv)
    D3 = o.eval(uv, 0x3C0).reshape(4, 3, n)
    D2 = lambda x: o.eval(x, 0x38).reshape(3, 3, n)  # noqa: E731  Suu, Suv, Svv
    eu = np.array([h, 0.0])
    ev = np.array([0.0, h])
    dU = (D2(uv + eu) - D2(uv - eu)) / (2 * h)
    dV = (D2(uv + ev) - D2(uv - ev)) / (2 * h)
    scale = np.abs(D3).max() + np.abs(dU).max()
    for got, fd in ((D3[0], dU[0]), (D3[1], dU[1]), (D3[1], dV[0]), (D3[2], dU[2]), (D3[2], dV[1]), (D3[3], dV[2])):
        assert np.abs(got - fd).max() <= 1e-6 * scale
    E = o.eval(uv, 6).reshape(2, 3, n)
    N = o.eval_normal(uv, 63).reshape(6, 3, n)
    assert np.abs(N[0] - np.cross(E[0].T, E[1].T).T).max() <= 1e-12 * np.abs(N[0]).max()
    Nf = lambda x: o.eval_normal(x, 7).reshape(3, 3, n)  # noqa: E731  N, Nu, Nv
    nU = (Nf(uv + eu) - Nf(uv - eu)) / (2 * h)
    nV = (Nf(uv + ev) - Nf(uv - ev)) / (2 * h)
    sc = np.abs(N).max()
    for got, fd in ((N[1], nU[0]), (N[2], nV[0]), (N[3], nU[1]), (N[4], nU[2]), (N[4], nV[1]), (N[5], nV[2])):
        assert np.abs(got - fd).max() <= 1e-6 * sc
    # a mask selects blocks in order
    sel = o.eval_normal(uv, 0b101000)
    assert np.array_equal(sel, np.concatenate([N[3], N[5]]))


def _projection_queries(o, n, seed, spread):
    """Points off the surface along its normal by up to +-spread/2 of the control net's extent,
    and points far from it (a box six extents wide)."""
    rng = np.random.default_rng(seed)
    uv = rng.random((n, 2))
    E = o.eval(uv, 7)
    N = np.cross(E[3:6].T, E[6:9].T)
    N /= np.linalg.norm(N, axis=1)[:, None]
    ext = np.ptp(o.cps, 0).max()
    near = E[0:3].T + N * ((rng.random(n) - 0.5) * spread * ext)[:, None]
    far = o.cps.mean(0) + (rng.random((n // 4, 3)) - 0.5) * 6 * ext
    return np.concatenate([near, far])


@pytest.mark.parametrize("kind", ["large", "small", "rational"])
def test_oracle_projection_is_a_constrained_minimum_and_mostly_global(kind):
    """The projection's answers: every query found; each answer a minimum of |S - P| over the
    closed domain (interior: gradient J^T r zero to rounding and Hessian positive definite; on an
    edge: the free derivative zero, the other pointing into the domain); and the global minimum
    (a 401x401 parameter grid) for at least 95 % of the queries."""
    from gpu_nurbs_gb300 import synth
    surf = {"large": synth.surface_large(), "small": synth.surface_small(),
            "rational": synth.surface_random(synth.Rng(77))}[kind]
    o = O.OracleSurface(surf)
    P = _projection_queries(o, 400, 5, 0.2)
    uv, st, res, _ = o.project(P)
    assert np.all(st <= O.FOUND_AMBIGUOUS)
    E = o.eval(uv, 63).reshape(6, 3, -1)
    r = E[0].T - P
    g = np.stack([(E[1].T * r).sum(1), (E[2].T * r).sum(1)], 1)
    scale = np.maximum(np.linalg.norm(r, axis=1), 1e-3) * np.maximum(np.linalg.norm(E[1], axis=0),
                                                                    np.linalg.norm(E[2], axis=0))
    ku = surf["knots_u"][surf["p"]], surf["knots_u"][surf["nu"]]
    kv = surf["knots_v"][surf["q"]], surf["knots_v"][surf["nv"]]
    for a, (lo, hi) in ((0, ku), (1, kv)):
        inner = (uv[:, a] > lo) & (uv[:, a] < hi)
        # 1e-6: a Newton step of 1e-10 ends the iteration, which leaves |g| ~ 1e-7 |r||J| in the
        # flat valleys of nearly degenerate minima
        assert np.all(np.abs(g[inner, a]) <= 1e-6 * scale[inner]), (a, np.abs(g[inner, a] / scale[inner]).max())
        assert np.all(g[uv[:, a] == lo, a] >= -1e-6 * scale[uv[:, a] == lo])
        assert np.all(g[uv[:, a] == hi, a] <= 1e-6 * scale[uv[:, a] == hi])
    interior = np.all((uv > [ku[0], kv[0]]) & (uv < [ku[1], kv[1]]), axis=1)
    h00 = (E[1] * E[1]).sum(0) + (r.T * E[3]).sum(0)
    h01 = (E[1] * E[2]).sum(0) + (r.T * E[4]).sum(0)
    h11 = (E[2] * E[2]).sum(0) + (r.T * E[5]).sum(0)
    det = h00 * h11 - h01 * h01
    assert np.all((h00[interior] > 0) & (det[interior] >= -1e-9 * (h00[interior] * h11[interior]))), kind
    gg = np.linspace(0, 1, 401)
    U, V = np.meshgrid(ku[0] + gg * (ku[1] - ku[0]), kv[0] + gg * (kv[1] - kv[0]), indexing="ij")
    G = o.eval(np.stack([U.ravel(), V.ravel()], 1), 1).T
    dmin = np.array([np.linalg.norm(G - x, axis=1).min() for x in P])
    assert np.mean(res <= dmin + 1e-12) >= 0.95, np.mean(res <= dmin + 1e-12)


def test_oracle_normal_cones_hold_the_sampled_normals():
    """Cones and bound boxes of the built nodes hold the normals and points sampled densely over
    each node's parameter rectangle (the lattice-plus-bound construction is not a proof); nodes
    whose cone is not every direction exist on the smooth surface."""
    from gpu_nurbs_gb300 import synth
    for surf in (synth.surface_small(), synth.surface_large()):
        o = O.OracleSurface(surf)
        t, _, b = o.tree()
        nb, cr, lat = o.cones()
        org = o.origin()
        g = (np.arange(17) + 0.5) / 17
        for k in np.nonzero(b)[0]:
            lo, hi = t[k, 0:2], t[k, 2:4]
            U, V = np.meshgrid(lo[0] + g * (hi[0] - lo[0]), lo[1] + g * (hi[1] - lo[1]), indexing="ij")
            uv = np.stack([U.ravel(), V.ravel()], 1)
            N = o.eval_normal(uv, 1).T
            S = o.eval(uv, 1).T - org
            assert np.all(S >= cr[k, 9:12] - 1e-12) and np.all(S <= cr[k, 12:15] + 1e-12), k
            assert np.all(N >= nb[k, :3] - 1e-9) and np.all(N <= nb[k, 3:] + 1e-9), k
            if cr[k, 7] > 0:
                c = (N @ cr[k, 4:7].astype(np.float64)) / np.linalg.norm(N, axis=1)
                assert np.all(c >= cr[k, 7] - 1e-6), (k, c.min(), cr[k, 7])
            Lk = o.eval(np.stack([np.repeat(lo[0] + np.arange(9) / 8 * (hi[0] - lo[0]), 9),
                                  np.tile(lo[1] + np.arange(9) / 8 * (hi[1] - lo[1]), 9)], 1), 1).T - org
            assert np.abs(lat[k] - Lk).max() <= 1e-6 * max(1.0, np.abs(Lk).max()), k
    assert np.any(O.OracleSurface(synth.surface_small()).cones()[1][:, 7] > 0)


def test_oracle_quadtree_inversion():
    """The adaptive quadtree inversion: points on the surface come back to 1e-12; points within
    max_edge of it are answered within max_edge; points far from the control net have no
    passing node (NO_CANDIDATE)."""
    from gpu_nurbs_gb300 import synth
    for surf in (synth.surface_small(), synth.surface_large(), tube(24, 8)):
        o = O.OracleSurface(surf)
        rng = np.random.default_rng(2)
        uv0 = rng.random((1000, 2))
        E = o.eval(uv0, 7)
        uv, st, res, _ = o.invert_quadtree(E[0:3].T, 1e-3)
        assert np.all(st <= O.FOUND_AMBIGUOUS)
        assert np.abs(res).max() <= 1e-12
        N = np.cross(E[3:6].T, E[6:9].T)
        N /= np.linalg.norm(N, axis=1)[:, None]
        P = E[0:3].T + N * ((rng.random(1000) - 0.5) * 1e-3)[:, None]
        uv, st, res, _ = o.invert_quadtree(P, 1e-3)
        assert np.mean(st <= O.FOUND_AMBIGUOUS) >= 0.99 and np.all(res[st <= 1] < 1e-3)
        far = o.cps.max(0) + 1.0 + rng.random((50, 3))
        assert np.all(o.invert_quadtree(far, 1e-3)[1] == O.NO_CANDIDATE)


PIN_FILES = sorted(glob.glob(os.path.join(GOLDEN, "pin3_*.npz")))


def _pin_surface(path):
    g = load_golden(os.path.join(GOLDEN, os.path.basename(path)[len("pin3_"):]))
    return surf_of(g), np.load(path)


@pytest.mark.parametrize("path", PIN_FILES, ids=lambda p: os.path.basename(p)[5:-4])
def test_oracle_third_order_pinned_to_reference(path):
    """The oracle's third-order and normal derivatives against the reference's own
    MatrixSurfaceRd* / new-style quotient forms / SurfaceNormalDerivative* (fixtures made by the
    reference compiled for the host): bit-identical for S, Su, Sv, Suu, Svv, Suuu, Svvv and N
    everywhere, and the mixed ones equal to rounding noise where the weights are constant; where
    they are not,
    the reference's S_uv, S_uuv, S_uvv carry its sign defect (the oracle's follow the quotient
    rule, checked against central differences elsewhere)."""
    surf, z = _pin_surface(path)
    o = O.OracleSurface(surf)
    mine = np.stack([np.concatenate([d, n[[0, 3, 4, 5]]]) for d, n in (o.ders3(u, v) for u, v in z["uv"])])
    ref = z["ders3"]
    exact_blocks = [0, 1, 2, 3, 5, 6, 9, 10]
    assert np.array_equal(mine[:, exact_blocks].view(np.int64), ref[:, exact_blocks].view(np.int64))
    if np.ptp(surf["weights"]) == 0:
        # constant weights: h's derivatives are rounding noise (~1e-17), so the defect's terms
        # change the mixed derivatives by ~1e-29 at most
        assert np.abs(mine - ref).max() <= 1e-20 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("path", PIN_FILES, ids=lambda p: os.path.basename(p)[5:-4])
def test_oracle_quadtree_pinned_to_reference(path):
    """The quadtree inversion's node tests against the reference's BoundingBoxCheck and
    getSplitType: box checks equal for every node and point; split types equal with the
    reference's v-length (MatrixSurfaceDerivativeU) reproduced; the oracle's own definition
    (the v-derivative) differs from it only where that length decides."""
    surf, z = _pin_surface(path)
    o = O.OracleSurface(surf)
    for e, me in enumerate(z["max_edge"]):
        for i, nd in enumerate(z["nodes"]):
            assert o.qt_split_type(nd, me, as_reference=True) == z["split"][e, i]
            for j, x in enumerate(z["P"]):
                assert o.qt_hull_check(nd, x, me) == z["box"][e, i, j]
