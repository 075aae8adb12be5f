"""GPU tests of the normal-cone build and nurbs_project (closest point over the closed domain)
against the oracle's restatement (oracle.OracleSurface.cones / .project)."""
import os

import numpy as np
import pytest

import oracle as O
from conftest import golden_files, load_golden
from parity import assert_exact, project_parity
from test_oracle import _projection_queries

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MODEL_FILES = [f for f in golden_files() if os.path.basename(f).startswith(("model_", "synth_"))]


def T(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def surfaces():
    from gpu_nurbs_gb300 import synth
    g = load_golden(MODEL_FILES[-1])
    model = dict(p=g["p"], q=g["q"], nu=g["nu"], nv=g["nv"], knots_u=g["knots_u"], knots_v=g["knots_v"],
                 cps=g["cps"], weights=g["weights"])
    return {"large": synth.surface_large(), "small": synth.surface_small(), "quintic": synth.surface_quintic(n=24),
            "rational": synth.surface_random(synth.Rng(77)), "model": model}


@pytest.mark.parametrize("which", ["large", "small", "quintic", "rational", "model"])
def test_normal_cones_bit_exact(nurbs, which):
    """Normal boxes, FP32 cone records and lattice points equal the oracle's bit for bit."""
    sf = surfaces()[which]
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    gb, gc, gl = s.normal_cones()
    ob, oc, ol = o.cones()
    _, _, built = o.tree()
    b = built.astype(bool)
    assert np.array_equal(gb[b].view(np.int64), ob[b].view(np.int64))
    assert np.array_equal(gc[b].view(np.int32), oc[b].view(np.int32))
    assert np.array_equal(gl[b].view(np.int32), ol[b].view(np.int32))


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("which", ["large", "small", "rational", "quintic"])
def test_project_parity(nurbs, which, precision):
    """Points up to 10 % of the extent off the surface along its normal and points far from it
    (a box six extents wide): every answer the oracle's, UNSTABLE queries (the oracle's own
    answer changes for perturbations at FP32 resolution) no farther than the farthest of its
    answers.  Mixed precision: FOUND_UNIQUE failures within the chaos bound of the mixed
    inversion."""
    sf = surfaces()[which]
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    P = _projection_queries(o, 4096, 11, 0.2)
    uv, st, res = (x.cpu().numpy() for x in s.project(T(P), precision))
    c = project_parity(o, P, uv, st, res)
    assert_exact(c, which, precision)
    assert np.all(st <= 1)


def test_project_on_the_surface_recovers_the_parameters(nurbs):
    """Points on the 64x64 surface: the projection returns their parameters (to 1e-9 where the
    minimum is unique) and is never farther than the inversion's answer."""
    from gpu_nurbs_gb300 import synth
    sf = synth.surface_large()
    s = nurbs.Surface(sf)
    o = O.OracleSurface(sf)
    uv0 = np.random.default_rng(4).random((8192, 2))
    P = o.eval(uv0, 1).T.copy()
    uv, st, res = (x.cpu().numpy() for x in s.project(T(P), nurbs.PREC_MIXED))
    assert np.all(st <= 1)
    assert res.max() <= 1e-12
    assert np.abs(uv - uv0)[st == 0].max() <= 1e-9
    iuv, ist, ires = (x.cpu().numpy() for x in s.invert(T(P), 0))
    found = ist <= 1
    assert np.all(res[found] <= ires[found] + 1e-14)


def test_project_edge_cases(nurbs):
    """Empty batches; a non-finite point (no candidate); points beyond the corners and edges of
    the domain (answers on the boundary); every answer inside the domain."""
    from gpu_nurbs_gb300 import synth
    sf = synth.surface_small()
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    s.project(T(np.zeros((0, 3))))
    E = o.eval(np.array([[0.0, 0.0], [1.0, 1.0], [0.0, 1.0], [1.0, 0.5], [0.5, 0.0]]), 7).reshape(3, 3, -1)
    out = E[0].T - 0.3 * E[1].T - 0.3 * E[2].T  # beyond the low-u, low-v side of each point
    P = np.concatenate([out, [[np.nan, 0.0, 0.0]]])
    uv, st, res = (x.cpu().numpy() for x in s.project(T(P)))
    assert st[-1] == nurbs.INV_NO_CANDIDATE
    assert np.all(st[:-1] <= 1)
    assert np.all((uv[:-1] >= 0) & (uv[:-1] <= 1))
    ouv, ost, ores, _ = o.project(P[:-1])
    assert np.abs(uv[:-1] - ouv).max() <= 1e-9
    assert np.all(np.abs(res[:-1] - ores) <= 1e-12 * ores + 1e-14)
    assert nurbs.lib().nurbs_project(s.h, None, 4, None, None, None, 0, None) == nurbs.E_INVALID
    assert nurbs.lib().nurbs_project(s.h, None, 0, None, None, None, 7, None) == nurbs.E_INVALID
    for prec in (0, 1):
        uv, st, res = (x.cpu().numpy() for x in s.project(T(P), prec))
        assert st[-1] == nurbs.INV_NO_CANDIDATE
        assert np.abs(uv[:-1] - ouv).max() <= 1e-9
