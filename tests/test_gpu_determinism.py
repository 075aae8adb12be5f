"""A query's inversion result does not depend on the other queries of its launch: the same
queries in generation order, reversed, and sorted by a spatial key (which changes which
queries share a warp and the order their seeds finish) give bit-identical results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def morton3(P, bits=10):
    lo, hi = P.min(0), P.max(0)
    q = ((P - lo) / np.maximum(hi - lo, 1e-300) * ((1 << bits) - 1)).astype(np.uint64)
    key = np.zeros(len(P), dtype=np.uint64)
    for b in range(bits):
        for d in range(3):
            key |= ((q[:, d] >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b + d)
    return key


def workload(nurbs, name, n, seed=21):
    from gpu_nurbs_gb300 import synth
    surf, kind = {"large": (synth.surface_large(), "large"), "small": (synth.surface_small(), "small"),
                  "quintic": (synth.surface_quintic(n=64), "small")}[name]
    s = nurbs.Surface(surf)
    uv, off = synth.query_params(n, seed, kind)
    E = s.eval(torch.as_tensor(uv, device="cuda"), nurbs.S | nurbs.SU | nurbs.SV).cpu().numpy()
    return s, synth.form_queries(E[0:3].T, E[3:6].T, E[6:9].T, off)


@pytest.mark.parametrize("name", ["large", "small", "quintic"])
@pytest.mark.parametrize("precision", [1, 0], ids=["mixed", "fp64"])
def test_inversion_independent_of_query_order(nurbs, name, precision):
    n = (1 << 16) if precision == 1 else (1 << 13)
    s, P = workload(nurbs, name, n)
    perms = [np.arange(n), np.arange(n)[::-1].copy(), np.argsort(morton3(P), kind="stable")]
    ref = None
    for perm in perms:
        uv, st, res = (x.cpu().numpy() for x in s.invert(torch.as_tensor(P[perm], device="cuda"), precision))
        got = [np.empty_like(uv), np.empty_like(st), np.empty_like(res)]
        got[0][perm], got[1][perm], got[2][perm] = uv, st, res
        if ref is None:
            ref = got
            continue
        assert np.array_equal(got[1], ref[1])
        assert np.array_equal(got[0], ref[0], equal_nan=True)
        assert np.array_equal(got[2], ref[2], equal_nan=True)
