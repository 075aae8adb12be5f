"""Edge cases of the CUDA path against the oracle: every degree pair the kernels dispatch
differently (the compiled (2,2), (3,3), (5,5) and the generic path, up to degree 7 and down to
bilinear), parameters outside the domain and on knots, queries that are NaN, infinite or far
from every box, and launch sizes around the warp and tail-chunk boundaries."""
import os

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN
from parity import assert_exact, classify_inversion, eval_errors, oracle_parity

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def T(x, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")


def surface(p, q, nu, nv, seed):
    from gpu_nurbs_gb300 import synth
    r = synth.Rng(seed)
    ku = synth.gapped_knots(p, nu, r)
    kv = synth.uniform_knots(q, nv)
    x = np.repeat(np.arange(nu) / (nu - 1), nv)
    y = np.tile(np.arange(nv) / (nv - 1), nu)
    z = 0.15 * np.sin(3 * x + 2 * y) + 0.05 * r.normal(nu * nv, 1.0)
    return dict(p=p, q=q, nu=nu, nv=nv, knots_u=ku, knots_v=kv, cps=np.stack([x, y, z], 1),
                weights=r.uniform(nu * nv, 0.5, 2.0))


DEGREES = [(1, 1), (2, 2), (3, 3), (5, 5), (2, 5), (7, 7), (7, 3)]


def queries(o, n, seed, sigma=1e-3):
    from gpu_nurbs_gb300 import synth
    rng = np.random.default_rng(seed)
    uv = rng.random((n, 2))
    E = o.eval(uv, 7)
    return synth.form_queries(E[0:3].T, E[3:6].T, E[6:9].T, rng.normal(0, sigma, n))


@pytest.mark.parametrize("pq", DEGREES, ids=lambda d: f"p{d[0]}q{d[1]}")
def test_degrees_eval_and_invert(nurbs, pq):
    p, q = pq
    sf = surface(p, q, max(p + 1, 9), max(q + 1, 7), 100 + 10 * p + q)
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    rng = np.random.default_rng(1)
    uv = rng.random((300, 2))
    uv[:4] = [[0, 0], [1, 1], [0, 1], [1, 0]]                  # domain corners
    uv[4:4 + 5, 0] = sf["knots_u"][p + 1:p + 6] if sf["nu"] > p + 5 else 0.5   # on interior knots
    ev = s.eval(T(uv), 63).cpu().numpy()
    errs = eval_errors(ev, o.eval(uv, 63))
    if max(p, q) <= 3:
        assert max(errs) <= 1e-12
    # residuals can differ by as much as the two FP64 evaluations of S do (degree 7: ~1e-13)
    res_abs = max(1e-14, 4 * errs[0])
    P = queries(o, 256, 2)
    for prec in (0, 1):
        g_uv, g_st, g_res = (x.cpu().numpy() for x in s.invert(T(P), prec))
        assert_exact(oracle_parity(o, P, g_uv, g_st, g_res, res_abs=res_abs), (pq, prec), prec)


def test_parameters_outside_the_domain_follow_find_span(nurbs):
    """findSpan clamps to the first/last span, so S extrapolates that span's polynomial."""
    sf = surface(3, 3, 8, 8, 7)
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    uv = np.array([[-0.1, 0.5], [1.1, 0.5], [0.5, -0.05], [0.5, 1.2], [-0.2, 1.3]])
    assert max(eval_errors(s.eval(T(uv), 63).cpu().numpy(), o.eval(uv, 63))) <= 1e-12


def test_nan_infinite_and_far_queries(nurbs):
    sf = surface(3, 3, 8, 8, 8)
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    P = np.array([[np.nan, 0.5, 0.0], [0.5, np.inf, 0.0], [-np.inf, 0.5, 0.1], [10.0, 10.0, 10.0],
                  [0.5, 0.5, -50.0]])
    for prec in (0, 1):
        uv, st, res = (x.cpu().numpy() for x in s.invert(T(P), prec))
        assert (st == nurbs.INV_NO_CANDIDATE).all(), st
        assert np.isnan(uv).all() and np.isnan(res).all()
    assert all(len(c) == 0 for c in o.candidates(P))


@pytest.mark.parametrize("n", [1, 31, 33, 4 * 152 * 4 * 4 * 32 + 13])
def test_launch_sizes(nurbs, n):
    """Sizes around a warp's 32 queries and, for the last one, the launch whose final rounds take
    small chunks: every query is answered, as it is when inverted on its own."""
    sf = surface(3, 3, 8, 8, 9)
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    P = queries(o, n, 3)
    uv, st, res = (x.cpu().numpy() for x in s.invert(T(P), 1))
    assert (st <= 1).mean() > 0.99
    pick = np.unique(np.concatenate([[0, n - 1], np.random.default_rng(4).integers(0, n, 64)]))
    u1, s1, r1 = (x.cpu().numpy() for x in s.invert(T(P[pick]), 1))
    assert np.array_equal(s1, st[pick]) and np.array_equal(u1, uv[pick], equal_nan=True)


def test_pool_generic_degrees_match_single_surface(nurbs):
    """Degree pairs without a compiled variant (bilinear, degree 7, mixed degrees) in one pool."""
    surfs = [surface(p, q, max(p + 1, 9), max(q + 1, 7), 200 + 10 * p + q) for p, q in DEGREES]
    pool = nurbs.Pool(1 << 28, max_surfaces=16)
    ids = pool.add(surfs)
    per = 64
    P = np.concatenate([queries(O.OracleSurface(sf), per, 5 + k) for k, sf in enumerate(surfs)])
    batch = nurbs.Batch(ids, np.arange(len(surfs) + 1) * per)
    for prec in (0, 1):
        for tile in (128, 16):
            pool.set_config(tile, 4)
            uv, st, res = (x.cpu().numpy() for x in pool.invert(batch, T(P), prec))
            for k, sf in enumerate(surfs):
                sl = slice(k * per, (k + 1) * per)
                u1, s1, r1 = (x.cpu().numpy() for x in nurbs.Surface(sf).invert(T(P[sl]), prec))
                assert np.array_equal(s1, st[sl]) and np.array_equal(u1, uv[sl], equal_nan=True), (k, prec, tile)


TRUTH = os.path.join(GOLDEN, "eval_truth.npz")


def truth_cases():
    z = np.load(TRUTH)
    return [tuple(int(x) for x in d) for d in z["degrees"]]


@pytest.mark.parametrize("pq", truth_cases(), ids=lambda d: f"p{d[0]}q{d[1]}")
def test_high_degree_eval_no_worse_than_reference(nurbs, pq):
    """Degrees 5 and 7: the power basis of the span matrices is ill-conditioned and FP64 errors
    reach 1e-11 relative in either formulation, so the bar is the reference's own accuracy:
    against 40-digit values of the surface (tests/golden/eval_truth.npz), this library's error
    per output block is at most twice the oracle's (plus 1e-14)."""
    z = np.load(TRUTH)
    tag = f"p{pq[0]}q{pq[1]}_"
    sf = {k: z[tag + k] for k in ("knots_u", "knots_v", "cps", "weights")}
    sf.update({k: int(z[tag + k]) for k in ("p", "q", "nu", "nv")})
    uv, truth = z[tag + "uv"], z[tag + "truth"]
    ev = nurbs.Surface(sf).eval(T(uv), 63).cpu().numpy()
    mine = eval_errors(ev, truth)
    ref = eval_errors(O.OracleSurface(sf).eval(uv, 63), truth)
    for b in range(6):
        assert mine[b] <= 2 * ref[b] + 1e-14, (b, mine, ref)


def test_host_buffer_pipeline_matches_device_call(nurbs):
    """Host-buffer inversion of a large batch equals the device-buffer call bit for bit, with
    pinned and with pageable host memory."""
    sf = surface(3, 3, 8, 8, 10)
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    n = (1 << 19) + 77
    P = queries(o, n, 6)
    uv, st, res = (x.cpu().numpy() for x in s.invert(T(P), 1))
    for pinned in (True, False):
        Ph = torch.from_numpy(P).pin_memory().numpy() if pinned else P.copy()
        out = tuple(torch.empty(sh, dtype=dt).pin_memory().numpy() if pinned else np.empty(sh, npdt)
                    for sh, dt, npdt in (((n, 2), torch.float64, np.float64), (n, torch.int32, np.int32),
                                         (n, torch.float64, np.float64)))
        hu, hs, hr = s.invert_host(Ph, 1, out=out)
        assert np.array_equal(hs, st) and np.array_equal(hu, uv, equal_nan=True) and np.array_equal(hr, res, equal_nan=True)


def test_one_surface_from_many_streams_and_threads(nurbs):
    """Inversions on one surface handle from four threads, each on its own stream, launched
    repeatedly and overlapping on the GPU: every result equals the serial one."""
    import threading
    import ctypes as C
    sf = surface(3, 3, 12, 12, 11)
    s, o = nurbs.Surface(sf), O.OracleSurface(sf)
    sets = [queries(o, 20000 + 37 * k, 20 + k) for k in range(4)]
    ref = [[x.cpu().numpy() for x in s.invert(T(P), 1)] for P in sets]
    streams = [torch.cuda.Stream() for _ in sets]
    inputs = [T(P) for P in sets]
    outs = [[None] * 6 for _ in sets]
    errors = []

    def work(k):
        try:
            h = C.c_void_p(streams[k].cuda_stream)
            for rep in range(6):
                outs[k][rep] = s.invert(inputs[k], 1, stream=h)
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(len(sets))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    torch.cuda.synchronize()
    assert not errors, errors
    for k in range(len(sets)):
        for rep in range(6):
            uv, st, res = (x.cpu().numpy() for x in outs[k][rep])
            assert np.array_equal(st, ref[k][1]) and np.array_equal(uv, ref[k][0], equal_nan=True), (k, rep)


def test_pcurve_of_a_curve_on_the_surface(nurbs):
    """p-curve extraction (the reference README's use of inversion): the samples of a 3-D curve
    lying on the surface, C(t) = S(u(t), v(t)) with (u, v) a closed loop in the domain, are
    inverted in one batch; the recovered parameters are the loop's to 1e-9 and consecutive
    samples stay close (no jumps between branches)."""
    from gpu_nurbs_gb300 import synth
    s = nurbs.Surface(synth.surface_large())
    t = np.linspace(0.0, 1.0, 4001)
    uv = np.stack([0.5 + 0.3 * np.cos(2 * np.pi * t), 0.5 + 0.2 * np.sin(4 * np.pi * t)], 1)
    C = s.eval(T(uv), nurbs.S).cpu().numpy().T.copy()         # (n, 3) samples of the curve
    for prec in (1, 0):
        g_uv, st, res = (x.cpu().numpy() for x in s.invert(T(C), prec))
        assert (st == nurbs.INV_FOUND).mean() > 0.999
        ok = st == nurbs.INV_FOUND
        assert np.abs(g_uv[ok] - uv[ok]).max() <= 1e-9
        assert res[ok].max() <= 1e-12
        step = np.abs(np.diff(g_uv, axis=0)).max(1)
        assert np.nanmax(step) < 5 * np.abs(np.diff(uv, axis=0)).max()


@pytest.mark.parametrize("offset", [(1000.0, -500.0, 250.0), (1e5, 2e5, -3e4)], ids=["1e3", "1e5"])
def test_translated_surface(nurbs, offset):
    """The same surface far from the origin (CAD coordinates): inversion still matches the
    oracle, and finds the same parameters as for the surface at the origin."""
    sf = surface(3, 3, 12, 12, 12)
    moved = dict(sf, cps=sf["cps"] + np.asarray(offset))
    o, om = O.OracleSurface(sf), O.OracleSurface(moved)
    P = queries(o, 2048, 13)
    Pm = P + np.asarray(offset)
    for prec in (1, 0):
        g_uv, g_st, g_res = (x.cpu().numpy() for x in nurbs.Surface(moved).invert(T(Pm), prec))
        assert_exact(oracle_parity(om, Pm, g_uv, g_st, g_res), (offset, prec), prec)
        b_uv, b_st, _ = (x.cpu().numpy() for x in nurbs.Surface(sf).invert(T(P), prec))
        both = (g_st == 0) & (b_st == 0)
        assert both.mean() > 0.95
        assert np.abs(g_uv[both] - b_uv[both]).max() <= 1e-6


@pytest.mark.parametrize("scale", [1e-3, 1e3], ids=["1e-3", "1e3"])
def test_scaled_surface(nurbs, scale):
    """The same surface in other units (metres vs millimetres): same parameters, oracle parity."""
    sf = surface(3, 3, 12, 12, 14)
    scaled = dict(sf, cps=sf["cps"] * scale)
    o, os_ = O.OracleSurface(sf), O.OracleSurface(scaled)
    P = queries(o, 2048, 15)
    Ps = P * scale
    for prec in (1, 0):
        g_uv, g_st, g_res = (x.cpu().numpy() for x in nurbs.Surface(scaled).invert(T(Ps), prec))
        assert_exact(oracle_parity(os_, Ps, g_uv, g_st, g_res), (scale, prec), prec)
        b_uv, b_st, _ = (x.cpu().numpy() for x in nurbs.Surface(sf).invert(T(P), prec))
        both = (g_st == 0) & (b_st == 0)
        assert both.mean() > 0.95
        assert np.abs(g_uv[both] - b_uv[both]).max() <= 1e-6
