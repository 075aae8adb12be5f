"""CPU tests of the C-ABI library: it loads, exports every declared symbol, and its host-only
entry points (.nu reader/writer, sizes, status strings) behave as the reference's readNu and
MatrixNPosition do.  No GPU compute is called here."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden_files, load_golden

HEADER = os.path.join(ROOT, "include", "gpu_nurbs.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nurbs_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(nurbs):
    L = nurbs.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    # and the Python binding declares a signature for each of them
    assert set(syms) <= set(nurbs.SIGNATURES)


def test_status_strings(nurbs):
    L = nurbs.lib()
    assert L.nurbs_status_string(0) == b"ok"
    assert L.nurbs_status_string(-5) == b"parse error"
    assert b"sm_103a" in L.nurbs_version()


def test_matrix_n_size_and_position(nurbs):
    L = nurbs.lib()
    # MatrixNPosition (src/NURBS/Evaluate.cu:110-112), sizes of src/main.cu:182
    p, q, nu, nv = 3, 2, 7, 9
    assert L.nurbs_matrix_n_size(p, q, nu, nv) == (p + nu) * (q + nv) * 4 * (p + 1) * (q + 1)
    for i, j, c in [(3, 2, 0), (4, 5, 3), (6, 8, 1)]:
        assert L.nurbs_matrix_n_position(i, j, p, q, nu, nv, c) == \
            i * (q + nv) * 4 * (p + 1) * (q + 1) + j * 4 * (p + 1) * (q + 1) + c * (p + 1) * (q + 1)


MODEL_FILES = [f for f in golden_files() if os.path.basename(f).startswith("model_")]


def nu_text(g, comments=True):
    """The .nu text of a fixture surface, in the layout of the reference's model files."""
    out = []
    if comments:
        out.append("** NURBS degree [2]")
    out.append(f"NU {g['p']} {g['q']}")
    out.append(f"CP {g['nu']} {g['nv']}")
    out.append("")
    out.append("** NURBS Knots")
    out.append("KNu " + " ".join(repr(float(x)) for x in g["knots_u"]))
    out.append("KNv " + " ".join(repr(float(x)) for x in g["knots_v"]))
    out.append("")
    for k in range(g["nu"] * g["nv"]):
        c = g["cps"][k]
        out.append("DP %r %r %r %r" % (float(c[0]), float(c[1]), float(c[2]), float(g["weights"][k])))
        if (k + 1) % g["nv"] == 0:
            out.append("")
    return "\n".join(out) + "\n"


@pytest.mark.parametrize("path", MODEL_FILES, ids=lambda p: os.path.basename(p)[:-4])
def test_nu_parse_matches_fixture(nurbs, path):
    g = load_golden(path)
    d = nurbs.parse_nu(nu_text(g))
    assert (d["p"], d["q"], d["nu"], d["nv"]) == (g["p"], g["q"], g["nu"], g["nv"])
    for k in ("knots_u", "knots_v", "cps", "weights"):
        assert np.array_equal(d[k], g[k]), k


def test_nu_write_read_round_trip(nurbs, tmp_path):
    g = load_golden(MODEL_FILES[0])
    path = str(tmp_path / "rt.nu")
    nurbs.write_nu(path, g)
    d = nurbs.read_nu(path)
    for k in ("knots_u", "knots_v", "cps", "weights"):
        assert np.array_equal(d[k], g[k]), k


@pytest.mark.parametrize("text", [
    "",                                   # no tags at all (the reference loops forever)
    "NU 3 3\n",                           # missing CP
    "NU 3 3\nCP 4 4\nKNu 0 0 0 0 1 1 1 1\n",   # missing KNv
    "NU 3 3\nCP 4 4\nKNu 0 0 0 0 1 1 1\nKNv 0 0 0 0 1 1 1 1\n",   # short knot line
    "NU 9 3\nCP 10 4\n",                  # degree above the supported maximum
    "NU 3 3\nCP 2 4\n",                   # net smaller than degree + 1
    "NU 1 1\nCP 2 2\nKNu 0 0 1 1\nKNv 0 0 1 1\nDP 0 0 0 1\nDP 0 1 0 1\nDP 1 0 0\n",  # short DP
    "NU 1 1\nCP 2 2\nKNu 0 0 1 1\nKNv 0 0 1 x\n",  # non-numeric
])
def test_nu_parse_errors(nurbs, text):
    with pytest.raises(nurbs.NurbsError) as e:
        nurbs.parse_nu(text)
    assert e.value.code in (nurbs.E_PARSE, nurbs.E_INVALID)


def test_nu_read_missing_file(nurbs, tmp_path):
    with pytest.raises(nurbs.NurbsError) as e:
        nurbs.read_nu(str(tmp_path / "none.nu"))
    assert e.value.code == nurbs.E_IO


def test_nu_comments_and_extra_values(nurbs):
    text = ("** header\nNU 1 1\n** x\nCP 2 2\nKNu 0 0 1 1 7 7\nKNv 0 0 1 1\nDP 0 0 0 1\n\n"
            "junk line\nDP 0 1 0 1\nDP 1 0 0 1\nDP 1 1 1 2\n")
    d = nurbs.parse_nu(text)
    assert np.array_equal(d["knots_u"], [0, 0, 1, 1])
    assert d["weights"][3] == 2.0


def test_pool_surface_bytes_admission_size(nurbs):
    """Host-only sizing used for budget admission: covers both span tables (FP64 and the FP32
    table padded to an even coefficient count per span), grows with the net, rejects bad input."""
    from gpu_nurbs_gb300 import synth
    small, large = synth.surface_small(), synth.surface_large()
    b_small, b_large = nurbs.surface_bytes(small), nurbs.surface_bytes(large)
    spans = lambda k, p: len(np.unique(k[p:len(k) - p]))  - 1
    for sf, b in ((small, b_small), (large, b_large)):
        p, q = sf["p"], sf["q"]
        ns = spans(sf["knots_u"], p) * spans(sf["knots_v"], q)
        k12 = (p + 1) * (q + 1)
        assert b >= ns * (k12 * 32 + (k12 + (k12 & 1)) * 16)
        assert b % 256 == 0
    assert b_large > b_small
    # degree 2 x 2: 9 coefficients per span, FP32 spans padded to 10
    d = dict(small, p=2, q=2, knots_u=synth.uniform_knots(2, small["nu"]), knots_v=synth.uniform_knots(2, small["nv"]))
    ns = (small["nu"] - 2) * (small["nv"] - 2)
    assert nurbs.surface_bytes(d) >= ns * (9 * 32 + 10 * 16)
    bad = dict(small, knots_u=small["knots_u"][::-1].copy())
    with pytest.raises(nurbs.NurbsError):
        nurbs.surface_bytes(bad)


def test_product_does_not_use_the_oracle():
    """The library and its binding never reach the oracle (test infrastructure only): no
    import, path or symbol of it in the package sources or the public headers."""
    import glob
    files = glob.glob(os.path.join(ROOT, "gpu-nurbs_gb300", "*.py")) + \
        glob.glob(os.path.join(ROOT, "gpu-nurbs_gb300", "csrc", "*")) + glob.glob(os.path.join(ROOT, "include", "*"))
    assert files
    for f in files:
        text = open(f, errors="replace").read()
        assert "import oracle" not in text and "orc_" not in text and "liboracle" not in text, f
