"""GPU parity tests: every stage of the CUDA path through the C-ABI against the golden
fixtures (made by the reference's own code) and the oracle."""
import os

import numpy as np
import pytest

import oracle as O
from conftest import golden_files, load_golden
from parity import assert_exact, classify_inversion, eval_errors, oracle_parity

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

MODEL_FILES = [f for f in golden_files() if os.path.basename(f).startswith(("model_", "synth_"))]


def surf_of(g):
    return dict(p=g["p"], q=g["q"], nu=g["nu"], nv=g["nv"], knots_u=g["knots_u"], knots_v=g["knots_v"],
                cps=g["cps"], weights=g["weights"])


@pytest.fixture(scope="module")
def cuda():
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    return torch.device("cuda:0")


def T(x, dev, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device=dev)


ids = lambda p: os.path.basename(p)[:-4]


def ref_hits_empty_span(g):
    """True when the reference's findSpan returns an empty span at a domain end (a knot of
    multiplicity > p+1 there, as in model/test.nu): the reference then divides 0/0 and reads an
    unwritten MatrixN slot, so its samples there are NaN; this library clamps to the nearest
    non-empty span instead.  Tree and inversion exactness are checked on the other models."""
    p, q, nu, nv = g["p"], g["q"], g["nu"], g["nv"]
    ku, kv = g["knots_u"], g["knots_v"]
    return ku[p] == ku[p + 1] or ku[nu - 1] == ku[nu] or kv[q] == kv[q + 1] or kv[nv - 1] == kv[nv]


CLEAN_FILES = [f for f in MODEL_FILES if not ref_hits_empty_span(load_golden(f))]


@pytest.mark.parametrize("path", MODEL_FILES, ids=ids)
def test_matrix_n_bit_exact(nurbs, cuda, path):
    g = load_golden(path)
    s = nurbs.Surface(surf_of(g))
    M = s.matrix_n().cpu().numpy()
    assert np.array_equal(M.view(np.int64), g["matrix_n"].view(np.int64))


@pytest.mark.parametrize("path", MODEL_FILES, ids=ids)
def test_legacy_get_matrix_n_raw_bit_exact(nurbs, cuda, path):
    g = load_golden(path)
    M = nurbs.get_matrix_n_raw(g["p"], g["q"], g["nu"], g["nv"], T(g["knots_u"], cuda), T(g["knots_v"], cuda),
                               T(g["cps"].reshape(-1), cuda), T(g["weights"], cuda)).cpu().numpy()
    assert np.array_equal(M.view(np.int64), g["matrix_n"].view(np.int64))


@pytest.mark.parametrize("path", MODEL_FILES, ids=ids)
def test_eval_within_1e12(nurbs, cuda, path):
    g = load_golden(path)
    s = nurbs.Surface(surf_of(g))
    ev = s.eval(T(g["uv"], cuda), 63).cpu().numpy()
    errs = eval_errors(ev, g["eval"])
    assert max(errs) <= 1e-12, errs


@pytest.mark.parametrize("path", MODEL_FILES, ids=ids)
def test_eval_exact_bit_exact(nurbs, cuda, path):
    """NURBS_PREC_EXACT evaluation equals the reference's own FP64 functions bit for bit (the
    golden fixtures), degree 5 models included."""
    g = load_golden(path)
    s = nurbs.Surface(surf_of(g))
    ev = s.eval(T(g["uv"], cuda), 63, precision=nurbs.PREC_EXACT).cpu().numpy()
    ref = g["eval"]
    ok = np.isfinite(ref)
    assert np.array_equal(ev[ok].view(np.int64), ref[ok].view(np.int64))


@pytest.mark.parametrize("which", ["quintic", "deg7"])
def test_eval_exact_high_degree_matches_the_oracle(nurbs, cuda, which):
    """At degrees 5 and 7, where the Horner path differs from the reference's formulation by the
    power basis's conditioning, NURBS_PREC_EXACT equals the oracle (the reference's expressions)
    bit for bit, also at span boundaries and domain corners."""
    from gpu_nurbs_gb300 import synth
    if which == "quintic":
        surf = synth.surface_quintic(n=32)
    else:
        r = np.random.default_rng(3)
        nu = nv = 12
        surf = dict(p=7, q=7, nu=nu, nv=nv, knots_u=synth.uniform_knots(7, nu), knots_v=synth.uniform_knots(7, nv),
                    cps=np.stack([np.repeat(np.linspace(0, 1, nu), nv), np.tile(np.linspace(0, 1, nv), nu),
                                  0.1 * r.standard_normal(nu * nv)], 1), weights=r.uniform(0.5, 2, nu * nv))
    o = O.OracleSurface(surf)
    rng = np.random.default_rng(4)
    uv = rng.random((4096, 2))
    ku = np.unique(surf["knots_u"])
    uv[:64, 0] = rng.choice(ku, 64)
    uv[64:68] = [[0, 0], [0, 1], [1, 0], [1, 1]]
    s = nurbs.Surface(surf)
    ev = s.eval(T(uv, cuda), 63, precision=nurbs.PREC_EXACT).cpu().numpy()
    assert np.array_equal(ev.view(np.int64), o.eval(uv, 63).view(np.int64))
    with pytest.raises(nurbs.NurbsError):
        s.eval(T(uv, cuda), 64, precision=nurbs.PREC_EXACT)


@pytest.mark.parametrize("mask", [1, 7, 2, 9, 32, 63])
def test_eval_masks(nurbs, cuda, mask):
    g = load_golden(MODEL_FILES[-1])
    s = nurbs.Surface(surf_of(g))
    full = s.eval(T(g["uv"], cuda), 63).cpu().numpy()
    part = s.eval(T(g["uv"], cuda), mask).cpu().numpy()
    rows = [r for b in range(6) if mask >> b & 1 for r in range(3 * b, 3 * b + 3)]
    assert np.array_equal(part, full[rows])


@pytest.mark.parametrize("path", MODEL_FILES, ids=ids)
def test_legacy_evaluate_random_bit_exact(nurbs, cuda, path):
    g = load_golden(path)
    xyz = nurbs.evaluate_random(T(g["uv"], cuda), T(g["matrix_n"], cuda), g["p"], g["q"], g["nu"], g["nv"],
                                T(g["knots_u"], cuda), T(g["knots_v"], cuda)).cpu().numpy()
    assert np.array_equal(xyz.T, g["eval"][0:3], equal_nan=True)


@pytest.mark.parametrize("path", CLEAN_FILES, ids=ids)
def test_tree_bit_exact(nurbs, cuda, path):
    g = load_golden(path)
    s = nurbs.Surface(surf_of(g))
    nodes, div, built = s.tree()
    assert np.array_equal(built, g["built"])
    b = built == 1
    assert np.array_equal(nodes[b], g["tree"][b], equal_nan=True)
    assert np.array_equal(div[b], g["divided"][b])


@pytest.mark.parametrize("path", CLEAN_FILES, ids=ids)
def test_candidates_bit_exact(nurbs, cuda, path):
    g = load_golden(path)
    s = nurbs.Surface(surf_of(g))
    lst, cnt = s.candidates(T(g["P"], cuda))
    lst, cnt = lst.cpu().numpy(), cnt.cpu().numpy()
    assert np.array_equal(cnt, g["cand_counts"])
    flat = np.concatenate([lst[k, :cnt[k]] for k in range(len(cnt))])
    assert np.array_equal(flat, g["cand_flat"])


def _config_surfaces(which):
    from gpu_nurbs_gb300 import synth
    if which == "large":
        return [synth.surface_large()]
    if which == "quintic":
        return [synth.surface_quintic()]
    return synth.batched_surfaces(64)[0]


@pytest.mark.parametrize("which", ["large", "quintic", "batched64"])
def test_tree_and_candidates_at_config_scale(nurbs, cuda, which):
    """Tree boxes, Divided flags and candidate lists bit-exact against the oracle on the
    workload surfaces (64x64 bicubic, 256x256 quintic, 64 surfaces of the batched workload),
    with queries near the surface and queries placed exactly on box faces and corners, where
    the kernel's FP32 prefilter hands the decision to the FP64 comparison."""
    surfs = _config_surfaces(which)
    nq = 4096 if len(surfs) == 1 else 256
    for k, sf in enumerate(surfs):
        o, s = O.OracleSurface(sf), nurbs.Surface(sf)
        on, od, ob = o.tree()
        nodes, div, built = s.tree()
        assert np.array_equal(built, ob), (which, k)
        b = ob == 1
        assert np.array_equal(nodes[b].view(np.int64), on[b].view(np.int64)), (which, k)
        assert np.array_equal(div[b], od[b]), (which, k)
        _, _, P = _queries(sf, nq, 40 + k, "large")
        # points on the faces and corners of the built boxes (lb/rt columns 4..6 / 7..9)
        rng = np.random.default_rng(k)
        bi = np.nonzero(b)[0]
        face = []
        for t in rng.choice(bi, size=min(32, len(bi)), replace=False):
            lb, rt = on[t, 4:7], on[t, 7:10]
            inner = lb + rng.random(3) * (rt - lb)
            c = rng.integers(0, 3)
            for end in (lb, rt):
                p_ = inner.copy()
                p_[c] = end[c]
                face.append(p_)
            face.append(np.where(rng.random(3) < 0.5, lb, rt))
        P = np.concatenate([P, np.array(face)])
        lst, cnt = s.candidates(T(P, cuda))
        lst, cnt = lst.cpu().numpy(), cnt.cpu().numpy()
        ref = o.candidates(P)
        assert np.array_equal(cnt, [len(r) for r in ref]), (which, k)
        for q in range(len(P)):
            assert np.array_equal(lst[q, :cnt[q]], ref[q]), (which, k, q)


def _queries(surf, n, seed, kind):
    from gpu_nurbs_gb300 import synth
    o = O.OracleSurface(surf)
    uv, off = synth.query_params(n, seed, kind)
    E = o.eval(uv, 7)
    return o, uv, synth.form_queries(E[0:3].T, E[3:6].T, E[6:9].T, off)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_invert_small_parity(nurbs, cuda, precision):
    from gpu_nurbs_gb300 import synth
    surf = synth.surface_small()
    o, uv_true, P = _queries(surf, 4000, 5, "small")
    s = nurbs.Surface(surf)
    uv, st, res = (x.cpu().numpy() for x in s.invert(T(P, cuda), precision))
    c = oracle_parity(o, P, uv, st, res)
    print("small", precision, {k: v for k, v in c.items() if k != "fail_idx"})
    assert_exact(c, "small", precision)
    assert c["same"] >= 0.95 * c["unique"]
    ok = st == 0
    assert np.abs(uv[ok] - uv_true[ok]).max() <= 1e-9


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_invert_large_parity(nurbs, cuda, precision):
    """The 64x64 bicubic workload (offsets |N(0,1e-2)|), 16,384 queries: no failure in any
    class (mixed precision: see parity.MIXED_CHAOS_FRAC); UNSTABLE queries (answers that the
    oracle's own FP32-resolution variants change) under 1 %."""
    from gpu_nurbs_gb300 import synth
    surf = synth.surface_large()
    o, uv_true, P = _queries(surf, 16384, 6, "large")
    s = nurbs.Surface(surf)
    uv, st, res = (x.cpu().numpy() for x in s.invert(T(P, cuda), precision))
    c = oracle_parity(o, P, uv, st, res)
    print("large", precision, {k: v for k, v in c.items() if k != "fail_idx"})
    assert_exact(c, "large", precision)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_invert_quintic_parity(nurbs, cuda, precision):
    """The degree-5 256x256 workload, 16,384 queries, with the parameter error of the matching
    queries against the oracle (max) bounded."""
    from gpu_nurbs_gb300 import synth
    surf = synth.surface_quintic()
    o, uv_true, P = _queries(surf, 16384, 7, "small")
    s = nurbs.Surface(surf)
    uv, st, res = (x.cpu().numpy() for x in s.invert(T(P, cuda), precision))
    # residuals can differ by as much as the two FP64 evaluations of S do at degree 5
    ev = s.eval(T(uv_true, cuda), 1).cpu().numpy()
    res_abs = max(1e-14, 4 * eval_errors(ev, o.eval(uv_true, 1))[0])
    c = oracle_parity(o, P, uv, st, res, res_abs=res_abs)
    print("quintic", precision, {k: v for k, v in c.items() if k != "fail_idx"})
    assert_exact(c, "quintic", precision)
    assert c["max_uv_err_same"] <= 1e-9


@pytest.mark.parametrize("path", CLEAN_FILES, ids=ids)
def test_invert_models_parity(nurbs, cuda, path):
    g = load_golden(path)
    surf = surf_of(g)
    o = O.OracleSurface(surf)
    P = g["P"]
    ouv, ost, ores, _ = o.invert(P)
    s = nurbs.Surface(surf)
    for precision in (0, 1):
        uv, st, res = (x.cpu().numpy() for x in s.invert(T(P, cuda), precision))
        c = classify_inversion(uv, st, res, ouv, ost, ores, P)
        print(os.path.basename(path), precision, {k: v for k, v in c.items() if k != "fail_idx"})
        for k in c["fail_idx"][:4]:
            print("  fail", k, P[k], "gpu", uv[k], st[k], res[k], "oracle", ouv[k], ost[k], ores[k])
        assert c["fail_no_candidate"] == 0, c
        assert c["fail_unique"] + c["fail_ambiguous"] == 0, c


def test_invert_host_matches_device(nurbs, cuda):
    from gpu_nurbs_gb300 import synth
    surf = synth.surface_small()
    _, _, P = _queries(surf, 1000, 9, "small")
    s = nurbs.Surface(surf)
    uv, st, res = (x.cpu().numpy() for x in s.invert(T(P, cuda), 1))
    huv, hst, hres = s.invert_host(P, 1)
    assert np.array_equal(uv, huv, equal_nan=True) and np.array_equal(st, hst)
    assert np.array_equal(res, hres, equal_nan=True)


def test_eval_f32_close(nurbs, cuda):
    from gpu_nurbs_gb300 import synth
    surf = synth.surface_large()
    o = O.OracleSurface(surf)
    uv = np.random.default_rng(1).random((4096, 2))
    ref = o.eval(uv, 63)
    s = nurbs.Surface(surf)
    ev = s.eval_f32(T(uv, cuda, torch.float32), 63).cpu().numpy().astype(np.float64)
    errs = eval_errors(ev, ref)
    # FP32 contraction of FP32-rounded span matrices: ~1e-6 on points, derivatives lose a
    # further factor to cancellation in the power basis
    assert errs[0] < 1e-5, errs
    assert max(errs[1:3]) < 2e-4, errs
    assert max(errs[3:]) < 5e-3, errs


def _block_errors(ev, ref):
    """Max error per 3-row block relative to the block's largest reference norm."""
    out = []
    for b in range(ref.shape[0] // 3):
        r = ref[3 * b:3 * b + 3]
        x = ev[3 * b:3 * b + 3]
        out.append(float(np.linalg.norm(x - r, axis=0).max() / max(np.linalg.norm(r, axis=0).max(), 1e-300)))
    return out


def _third_order_cases():
    from gpu_nurbs_gb300 import synth
    return {"large": synth.surface_large(), "quintic": synth.surface_quintic(n=24),
            "rational": synth.surface_random(synth.Rng(77)), "model": surf_of(load_golden(MODEL_FILES[-1]))}


@pytest.mark.parametrize("which", ["large", "quintic", "rational", "model"])
def test_eval_third_order_and_normals(nurbs, cuda, which):
    """Third derivatives (mask bits 64..512) and the normal with its derivatives against the
    oracle's power-vector restatement, including the span boundaries and the domain corners:
    within 1e-11 of each block's magnitude (the fast path contracts in Horner form)."""
    surf = _third_order_cases()[which]
    o = O.OracleSurface(surf)
    rng = np.random.default_rng(9)
    ku = np.unique(surf["knots_u"][surf["p"]:surf["nu"] + 1])
    kv = np.unique(surf["knots_v"][surf["q"]:surf["nv"] + 1])
    uv = rng.random((8192, 2)) * [ku[-1] - ku[0], kv[-1] - kv[0]] + [ku[0], kv[0]]
    uv[:64, 0] = rng.choice(ku, 64)
    uv[64:128, 1] = rng.choice(kv, 64)
    uv[128:132] = [[ku[0], kv[0]], [ku[0], kv[-1]], [ku[-1], kv[0]], [ku[-1], kv[-1]]]
    s = nurbs.Surface(surf)
    ev = s.eval(T(uv, cuda), 1023).cpu().numpy()
    ref = o.eval(uv, 1023)
    errs = _block_errors(ev, ref)
    assert max(errs) <= 1e-11, errs
    part = s.eval(T(uv, cuda), 0b1010000000).cpu().numpy()
    assert np.array_equal(part, ev[np.r_[21:24, 27:30]])
    nv = s.eval_normal(T(uv, cuda), 63).cpu().numpy()
    errs = _block_errors(nv, o.eval_normal(uv, 63))
    assert max(errs) <= 1e-11, errs
    assert np.array_equal(s.eval_normal(T(uv, cuda), 0b100100).cpu().numpy(), nv[np.r_[6:9, 15:18]])


def test_invalid_arguments_return_status(nurbs, cuda):
    g = load_golden(MODEL_FILES[0])
    bad = surf_of(g)
    bad["weights"] = g["weights"].copy()
    bad["weights"][0] = np.nan
    with pytest.raises(nurbs.NurbsError) as e:
        nurbs.Surface(bad)
    assert e.value.code == nurbs.E_INVALID
    bad = surf_of(g)
    bad["knots_u"] = g["knots_u"][::-1].copy()
    with pytest.raises(nurbs.NurbsError) as e:
        nurbs.Surface(bad)
    assert e.value.code == nurbs.E_INVALID
    s = nurbs.Surface(surf_of(g))
    uv = T(g["uv"], cuda)
    with pytest.raises(nurbs.NurbsError):
        s.eval(uv, 0)
    with pytest.raises(nurbs.NurbsError):
        s.eval(uv, 1024)
    with pytest.raises(nurbs.NurbsError):
        s.eval_normal(uv, 64)
    with pytest.raises(nurbs.NurbsError):
        s.invert(T(g["P"], cuda), precision=7)
    # empty batches are valid no-ops
    s.eval(uv[:0], 1)
    s.invert(T(g["P"], cuda)[:0], 1)
    torch.cuda.synchronize()


def test_work_counter(nurbs, cuda):
    """The counting variant of the inversion kernel: deterministic counts, at least one seed
    iteration per candidate of a query and at most the cap per candidate, and one to three final
    FP64 polishes per query with an FP32 minimum (mixed)."""
    from gpu_nurbs_gb300 import synth
    surf = synth.surface_large()
    o, _, P = _queries(surf, 4096, 8, "large")
    s = nurbs.Surface(surf)
    cand = sum(len(c) for c in o.candidates(P))
    for precision in (0, 1):
        w1 = s.count_work(T(P, cuda), precision)
        w2 = s.count_work(T(P, cuda), precision)
        assert w1 == w2
        assert cand <= w1["seed_iterations"] <= 40 * cand
        if precision == 1:
            assert 0.9 * len(P) <= w1["final_polishes"] <= 3 * len(P)
        else:
            assert w1["final_polishes"] == 0
