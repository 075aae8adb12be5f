"""GPU parity tests: every stage of the CUDA path through the C-ABI against the golden
fixtures (made by the reference's own code) and the oracle."""
import os

import numpy as np
import pytest

import oracle as O
from conftest import golden_files, load_golden
from parity import classify_inversion, eval_errors

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
    ouv, ost, ores, _ = o.invert(P)
    s = nurbs.Surface(surf)
    uv, st, res = (x.cpu().numpy() for x in s.invert(T(P, cuda), precision))
    c = classify_inversion(uv, st, res, ouv, ost, ores, P)
    print("small", precision, {k: v for k, v in c.items() if k != "fail_idx"})
    assert c["fail_unique"] == 0 and c["fail_ambiguous"] == 0 and c["fail_no_candidate"] == 0, c
    assert c["same"] >= 0.95 * c["unique"]
    ok = st == 0
    assert np.abs(uv[ok] - uv_true[ok]).max() <= 1e-9


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_invert_large_parity(nurbs, cuda, precision):
    from gpu_nurbs_gb300 import synth
    surf = synth.surface_large()
    o, uv_true, P = _queries(surf, 1500, 6, "large")
    ouv, ost, ores, _ = o.invert(P)
    s = nurbs.Surface(surf)
    uv, st, res = (x.cpu().numpy() for x in s.invert(T(P, cuda), precision))
    c = classify_inversion(uv, st, res, ouv, ost, ores, P)
    print("large", precision, {k: v for k, v in c.items() if k != "fail_idx"})
    assert c["fail_no_candidate"] == 0
    assert c["fail_unique"] + c["fail_ambiguous"] <= 0.01 * c["n"], c


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
        s.eval(uv, 64)
    with pytest.raises(nurbs.NurbsError):
        s.invert(T(g["P"], cuda), precision=7)
    # empty batches are valid no-ops
    s.eval(uv[:0], 1)
    s.invert(T(g["P"], cuda)[:0], 1)
    torch.cuda.synchronize()
