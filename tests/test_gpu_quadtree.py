"""GPU tests of nurbs_invert_quadtree (the adaptive quadtree inversion) against the oracle's
restatement (oracle.OracleSurface.invert_quadtree)."""
import numpy as np
import pytest

import oracle as O
from test_oracle import tube

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def T(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def cases():
    from gpu_nurbs_gb300 import synth
    return {"small": synth.surface_small(), "large": synth.surface_large(), "tube": tube(24, 8),
            "rational": synth.surface_random(synth.Rng(77)), "quintic": synth.surface_quintic(n=32)}


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("which", ["small", "large", "tube", "rational", "quintic"])
@pytest.mark.parametrize("max_edge", [1e-2, 1e-4])
def test_quadtree_matches_the_oracle(nurbs, which, max_edge, precision):
    """Points on the surface, within max_edge of it, and far from it: the same status, the same
    answer to 1e-9, the same residual to rounding.  Mixed: the root's FP32 trajectory can end in
    another basin than the FP64 one (large GN steps over a wavy surface); its answer is then
    another point within max_edge, which the reference's success test accepts as well: found /
    not found differs for at most 1e-4 of the queries, the answer for at most 1e-3."""
    sf = cases()[which]
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    rng = np.random.default_rng(7)
    uv0 = rng.random((4096, 2))
    E = o.eval(uv0, 7)
    N = np.cross(E[3:6].T, E[6:9].T)
    N /= np.linalg.norm(N, axis=1)[:, None]
    near = E[0:3].T + N * ((rng.random(4096) - 0.5) * max_edge)[:, None]
    far = o.cps.mean(0) + (rng.random((256, 3)) - 0.5) * 6 * np.ptp(o.cps, 0).max()
    P = np.concatenate([E[0:3].T, near, far])
    uv, st, res = (x.cpu().numpy() for x in s.invert_quadtree(T(P), max_edge, precision))
    ouv, ost, ores, _ = o.invert_quadtree(P, max_edge)
    same = (st == ost) & ((st > 1) | (np.abs(uv - ouv).max(1) <= 1e-9))
    if precision == 0:
        assert np.all(same), np.nonzero(~same)[0][:10]
    else:
        assert np.count_nonzero((st <= 1) != (ost <= 1)) <= int(np.ceil(1e-4 * len(P)))
        assert np.count_nonzero(~same) <= int(np.ceil(1e-3 * len(P))), np.nonzero(~same)[0][:10]
        assert np.all(res[(st <= 1) & ~same] < max_edge)
    f = (st <= 1) & same
    assert np.abs(uv[f] - ouv[f]).max() <= 1e-9
    assert np.all(np.abs(res[f] - ores[f]) <= 1e-12 * ores[f] + 1e-14)
    assert np.mean(st[:4096] <= 1) == 1.0


def test_quadtree_arguments(nurbs):
    from gpu_nurbs_gb300 import synth
    s = nurbs.Surface(synth.surface_small())
    P = T(np.zeros((4, 3)))
    with pytest.raises(nurbs.NurbsError):
        s.invert_quadtree(P, 0.0)
    with pytest.raises(nurbs.NurbsError):
        s.invert_quadtree(P, float("nan"))
    with pytest.raises(nurbs.NurbsError):
        s.invert_quadtree(P, 1e-3, 5)
    s.invert_quadtree(P[:0], 1e-3)


def test_quadtree_and_projection_on_concurrent_streams(nurbs):
    """The same surface on two streams at once (each call takes its own launch counter): the
    results equal those of the calls one after the other."""
    from gpu_nurbs_gb300 import synth
    sf = synth.surface_large()
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    uv0 = np.random.default_rng(12).random((50000, 2))
    P = T(o.eval(uv0, 1).T)
    ref_q = [x.cpu().numpy() for x in s.invert_quadtree(P, 1e-4, 1)]
    ref_p = [x.cpu().numpy() for x in s.project(P, 1)]
    torch.cuda.synchronize()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    outs = []
    for _ in range(3):
        s1.wait_stream(torch.cuda.current_stream())
        s2.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s1):
            a = s.invert_quadtree(P, 1e-4, 1)
        with torch.cuda.stream(s2):
            b = s.project(P, 1)
            c = s.invert_quadtree(P, 1e-4, 0)
        outs.append((a, b, c))
    torch.cuda.synchronize()
    ref_q64 = [x.cpu().numpy() for x in s.invert_quadtree(P, 1e-4, 0)]
    for a, b, c in outs:
        for x, y in zip(a, ref_q):
            assert np.array_equal(x.cpu().numpy(), y, equal_nan=True)
        for x, y in zip(b, ref_p):
            assert np.array_equal(x.cpu().numpy(), y, equal_nan=True)
        for x, y in zip(c, ref_q64):
            assert np.array_equal(x.cpu().numpy(), y, equal_nan=True)
