"""GPU tests of nurbs_pcurve (p-curves of 3-D curves on a surface) against the oracle's
restatement (oracle.OracleSurface.pcurve)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def T(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def loop(n, cu=0.5, cv=0.5, ru=0.3, rv=0.2):
    t = np.linspace(0.0, 1.0, n)
    return np.stack([cu + ru * np.cos(2 * np.pi * t), cv + rv * np.sin(4 * np.pi * t)], 1)


def compare(g, r, res_abs=1e-14):
    g_uv, g_st, g_res, g_fl = g
    o_uv, o_st, o_res, o_fl = r
    assert np.array_equal(g_st, o_st)
    assert np.array_equal(g_fl, o_fl)
    ok = o_st <= 1
    assert np.abs(g_uv[ok] - o_uv[ok]).max() <= 1e-9
    assert np.all(np.abs(g_res[ok] - o_res[ok]) <= 1e-12 * o_res[ok] + res_abs)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_pcurve_on_the_surface_matches_the_oracle(nurbs, precision):
    """A closed loop C(t) = S(u(t), v(t)) on the 64x64 surface, 4001 samples: the p-curve is the
    loop's parameters to 1e-9, no flags, and the same as the oracle's p-curve sample by sample."""
    from gpu_nurbs_gb300 import synth
    sf = synth.surface_large()
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    uv = loop(4001)
    C = o.eval(uv, 1).T.copy()
    g = [x.cpu().numpy() for x in s.pcurve(T(C), precision)]
    r = o.pcurve(C)
    compare(g, r)
    assert np.all(g[1] == nurbs.INV_FOUND) and np.all(g[3] == 0)
    assert np.abs(g[0] - uv).max() <= 1e-9


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_pcurve_near_the_surface(nurbs, precision):
    """Samples 1e-3 off the 64x64 surface along the normal: every sample matches the oracle's
    p-curve (parameters, status, residual, flags) and none is flagged."""
    from gpu_nurbs_gb300 import synth
    sf = synth.surface_large()
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    uv = loop(3001)
    E = o.eval(uv, 7)
    C = synth.form_queries(E[0:3].T, E[3:6].T, E[6:9].T, np.full(len(uv), 1e-3))
    g = [x.cpu().numpy() for x in s.pcurve(T(C), precision)]
    compare(g, o.pcurve(C))
    assert np.count_nonzero(g[3]) == 0


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_pcurve_seam_jump(nurbs, precision):
    """A curve around a closed tube crosses its seam (u = 1 meets u = 0): the parameter jumps
    while the curve does not, and that sample alone carries the jump flag, as in the oracle."""
    from test_oracle import tube
    sf = tube()
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    u = (0.3 + np.arange(300) / 250.0 + 0.5 / 250) % 1.0
    uv = np.stack([u, np.full(300, 0.4)], 1)
    C = o.eval(uv, 1).T.copy()
    g = [x.cpu().numpy() for x in s.pcurve(T(C), precision)]
    compare(g, o.pcurve(C))
    wrap = int(np.nonzero(np.diff(u) < 0)[0][0]) + 1
    assert g[3][wrap] & nurbs.PCURVE_JUMP and np.count_nonzero(g[3] & nurbs.PCURVE_JUMP) == 1


def test_pcurve_continuation_repairs_a_sample(nurbs):
    """A sample whose tree seeds find no minimum takes its neighbours' continuation: on the 8x8
    surface, samples far enough above a bump that the inversion alone fails still come out
    found and continuous; the oracle does the same."""
    from gpu_nurbs_gb300 import synth
    sf = synth.surface_small()
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    uv = loop(2001, 0.5, 0.5, 0.35, 0.35)
    E = o.eval(uv, 7)
    C = synth.form_queries(E[0:3].T, E[3:6].T, E[6:9].T, np.full(len(uv), 2e-2))
    g = [x.cpu().numpy() for x in s.pcurve(T(C), 0)]
    compare(g, o.pcurve(C))
    inv_st = s.invert(T(C), 0)[1].cpu().numpy()
    assert (g[1] <= 1).sum() >= (inv_st <= 1).sum()


def test_pcurve_arguments(nurbs):
    from gpu_nurbs_gb300 import synth
    s = nurbs.Surface(synth.surface_small())
    with pytest.raises(nurbs.NurbsError):
        s.pcurve(T(np.zeros((4, 3))), precision=7)
    out = s.pcurve(T(np.zeros((0, 3))), 1)
    assert out[0].shape == (0, 2)
