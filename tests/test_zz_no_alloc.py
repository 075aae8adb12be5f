"""GPU test of nurbs_get_matrix_n_noalloc, the GetMatrixN entry point that allocates nothing.

It exists for callers that cannot allocate device memory at conversion time (a host
application whose allocator owns the device memory, a budget admitter that forbids allocations
outside its pool, a serving loop that must not enter the allocator between requests).  Its
output must equal the allocating entry point nurbs_get_matrix_n_raw bit for bit — the
tolerance every span-matrix test uses — on consecutive calls, since all calls share one static
scratch array that keeps the previous call's contents.  Collected last (file name) so that a
run stopping at its first failure has already run every other test; it also passes alone in a
fresh process.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import golden_files, load_golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev(x):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")


def _call(nurbs, fn, g):
    n = nurbs.lib().nurbs_matrix_n_size(g["p"], g["q"], g["nu"], g["nv"])
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    args = (g["p"], g["q"], g["nu"], g["nv"], _dev(g["knots_u"]), _dev(g["knots_v"]),
            _dev(g["cps"].reshape(-1)), _dev(g["weights"]))
    keep = args[4:]
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = fn(out.data_ptr(), *args[:4], *(t.data_ptr() for t in keep), st)
    torch.cuda.synchronize()
    return rc, out.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice(nurbs):
    assert torch.cuda.is_available()
    L = nurbs.lib()
    files = [f for f in golden_files() if os.path.basename(f).startswith(("model_", "synth_"))]
    # two different surfaces back to back, then the first again: the shared scratch holds the
    # previous call's tables each time
    order = [files[0], files[-1], files[0]]
    for path in order:
        g = load_golden(path)
        rc_ref, ref = _call(nurbs, L.nurbs_get_matrix_n_raw, g)
        assert rc_ref == 0
        for _ in range(2):
            rc, got = _call(nurbs, L.nurbs_get_matrix_n_noalloc, g)
            assert rc == 0, nurbs.lib().nurbs_status_string(rc)
            assert np.array_equal(got.view(np.int64), ref.view(np.int64))


def test_noalloc_rejects_surfaces_beyond_the_scratch(nurbs):
    L = nurbs.lib()
    p = q = 7
    nu = nv = 2000   # worst case scratch far above 1 MiB
    ku = np.concatenate([np.zeros(p), np.linspace(0, 1, nu - p + 1), np.ones(p)])
    g = dict(p=p, q=q, nu=nu, nv=nv, knots_u=ku, knots_v=ku, cps=np.zeros((4, 3)), weights=np.ones(4))
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    t = _dev(ku)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.nurbs_get_matrix_n_noalloc(out.data_ptr(), p, q, nu, nv, t.data_ptr(), t.data_ptr(), t.data_ptr(),
                                      t.data_ptr(), st)
    assert rc == nurbs.E_UNSUPPORTED
    assert b"scratch" in nurbs.lib().nurbs_last_error()
