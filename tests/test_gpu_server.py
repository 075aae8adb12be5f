"""GPU tests of the serving loop: results are the same alone and in the mix, uploads convert into
the pool and can be queried, eviction keeps uploads admitted under the budget, waits are bounded."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def queries(surf, n, rng, sigma=2e-3):
    from gpu_nurbs_gb300 import synth
    o = O.OracleSurface(surf)
    uv = rng.random((n, 2))
    E = o.eval(uv, 7)
    return synth.form_queries(E[0:3].T, E[3:6].T, E[6:9].T, rng.normal(0, sigma, n))


def same_within_tolerance(a, b, P):
    """Status equal; where found, uv within 1e-12 and residual within 1e-14 max(1,|P|)."""
    (uva, sta, resa), (uvb, stb, resb) = a, b
    if not np.array_equal(sta, stb):
        return False
    ok = sta <= 1
    if not np.all(np.abs(uva[ok] - uvb[ok]) <= 1e-12):
        return False
    scale = np.maximum(np.abs(P[ok]).max(1), 1.0)
    return bool(np.all(np.abs(resa[ok] - resb[ok]) <= 1e-14 * scale))


@pytest.fixture(scope="module")
def served(nurbs):
    from gpu_nurbs_gb300 import synth
    surfs, _ = synth.batched_surfaces(12, seed=9)
    surfs = [synth.surface_small(), synth.surface_large()] + surfs
    pool = nurbs.Pool(1 << 30, max_surfaces=64)
    ids = pool.add(surfs)
    return surfs, pool, ids


def test_each_result_same_alone_and_in_the_mix(nurbs, served, request):
    surfs, pool, ids = served
    rng = np.random.default_rng(4)
    reqs = []
    for _ in range(64):
        k = int(rng.integers(len(surfs)))
        reqs.append((k, queries(surfs[k], int(rng.integers(1, 400)), rng)))
    srv = nurbs.Server(pool, slots=4, max_batch_queries=8192, precision=nurbs.PREC_MIXED)
    request.addfinalizer(srv.close)
    alone = []
    for k, P in reqs:
        t, out = srv.submit_invert(int(ids[k]), P)
        assert srv.wait(t) == 0
        alone.append(out[:3])
    tickets = [srv.submit_invert(int(ids[k]), P) for k, P in reqs]
    assert srv.drain() == 0
    bad = []
    for i, ((k, P), (t, out), a) in enumerate(zip(reqs, tickets, alone)):
        assert srv.wait(t) == 0
        if not same_within_tolerance(a, out[:3], P):
            d = np.nonzero((a[1] != out[1]) | (np.abs(a[0] - out[0]).max(1) > 1e-12))[0]
            bad.append((i, k, d[:3].tolist(), a[1][d[:3]].tolist(), out[1][d[:3]].tolist(),
                        a[0][d[:3]].tolist(), out[0][d[:3]].tolist()))
        assert out[3][0] > 0   # latency recorded
    assert not bad, bad
    st = srv.stats()
    assert st.completed == 128 and st.in_flight == 0
    assert st.batches < 128   # the mix was batched
    srv.close()


def test_upload_then_query(nurbs, served, request):
    from gpu_nurbs_gb300 import synth
    surfs, pool, ids = served
    new = synth.batched_surfaces(3, seed=77)[0][2]
    srv = nurbs.Server(pool, slots=2, max_batch_queries=4096)
    request.addfinalizer(srv.close)
    t, sid = srv.submit_upload(new)
    assert srv.wait(t) == 0 and sid[0] >= 0
    P = queries(new, 300, np.random.default_rng(1))
    t2, out = srv.submit_invert(int(sid[0]), P)
    assert srv.wait(t2) == 0
    ref = [x.cpu().numpy() for x in nurbs.Surface(new).invert(torch.as_tensor(P, device="cuda"), nurbs.PREC_MIXED)]
    assert np.array_equal(out[1], ref[1])
    ok = ref[1] <= 1
    assert np.abs(out[0][ok] - ref[0][ok]).max(initial=0) <= 1e-12
    srv.close()


def test_bounded_wait_and_pause(nurbs, served, request):
    surfs, pool, ids = served
    srv = nurbs.Server(pool, slots=1, max_batch_queries=1024)
    request.addfinalizer(srv.close)
    srv.pause(True)
    P = queries(surfs[0], 50, np.random.default_rng(2))
    t, out = srv.submit_invert(int(ids[0]), P)
    assert srv.wait(t, timeout_ms=50) == nurbs.E_TIMEOUT
    srv.pause(False)
    assert srv.wait(t, timeout_ms=10000) == 0
    assert srv.wait(12345678, timeout_ms=1) == nurbs.E_INVALID
    srv.close()


def test_uploads_evict_least_recently_used(nurbs, request):
    from gpu_nurbs_gb300 import synth
    surfs, _ = synth.batched_surfaces(24, seed=11)
    sizes = [nurbs.surface_bytes(s) for s in surfs]
    slot_bytes = 4 * (2048 * 52 + 1024)
    pool = nurbs.Pool(int(sum(sorted(sizes)[-4:]) + 2 * slot_bytes + (4 << 20)), max_surfaces=64)
    srv = nurbs.Server(pool, slots=1, max_batch_queries=2048)
    request.addfinalizer(srv.close)
    got = []
    for s in surfs:
        t, sid = srv.submit_upload(s)
        assert srv.wait(t) == 0, "upload refused although older surfaces were evictable"
        got.append(int(sid[0]))
    info = pool.info()
    assert info.surfaces < len(surfs) and info.used_bytes <= info.budget_bytes
    # the most recent upload is resident and can be queried
    P = queries(surfs[-1], 64, np.random.default_rng(3))
    t, out = srv.submit_invert(got[-1], P)
    assert srv.wait(t) == 0
    srv.close()


def test_queries_while_uploads_evict(nurbs, request):
    """Queries submitted while uploads force evictions: a query against a surface that is no longer
    resident is refused at submission; every accepted query completes with the results the same
    surface gives alone (an evicted surface is never released while a queued request uses it)."""
    from gpu_nurbs_gb300 import synth
    surfs, _ = synth.batched_surfaces(32, seed=13)
    sizes = [nurbs.surface_bytes(s) for s in surfs]
    slot_bytes = 4 * (4096 * 52 + 1024)
    pool = nurbs.Pool(int(sum(sorted(sizes)[-4:]) + 4 * slot_bytes + (4 << 20)), max_surfaces=64)
    srv = nurbs.Server(pool, slots=2, max_batch_queries=4096)
    request.addfinalizer(srv.close)
    rng = np.random.default_rng(5)
    ids, accepted, refused = [], [], 0
    for k, sf in enumerate(surfs):
        t, sid = srv.submit_upload(sf)
        for j in range(3):  # queries against recent surfaces while this upload may evict them
            if not ids:
                break
            pick = int(rng.integers(max(0, len(ids) - 4), len(ids)))
            P = queries(surfs[pick], int(rng.integers(16, 512)), rng)
            try:
                tq, out = srv.submit_invert(ids[pick], P)
                accepted.append((tq, pick, P, out))
            except nurbs.NurbsError:
                refused += 1
        assert srv.wait(t) == 0
        ids.append(int(sid[0]))
    for tq, pick, P, out in accepted:
        assert srv.wait(tq) == 0
        ref = [x.cpu().numpy() for x in nurbs.Surface(surfs[pick]).invert(torch.as_tensor(P, device="cuda"),
                                                                           nurbs.PREC_MIXED)]
        assert same_within_tolerance(out[:3], ref, P)
    assert len(accepted) > 0
    info = pool.info()
    assert info.surfaces < len(surfs)
    srv.close()


def test_replay_trace(nurbs, served, request):
    surfs, pool, ids = served
    rng = np.random.default_rng(6)
    nreq = 200
    sizes = rng.integers(1, 300, nreq)
    qoff = np.concatenate([[0], np.cumsum(sizes)])
    which = rng.integers(0, len(surfs), nreq)
    P = np.concatenate([queries(surfs[k], int(m), rng) for k, m in zip(which, sizes)])
    arrival = np.cumsum(rng.exponential(50.0, nreq))   # 20k requests/s
    srv = nurbs.Server(pool, slots=4, max_batch_queries=16384)
    request.addfinalizer(srv.close)
    uv, st, res, lat, results, _ = srv.replay(arrival, np.zeros(nreq), ids[which], qoff, P)
    assert np.all(results == 0)
    assert np.all(lat > 0) and np.percentile(lat, 50) < 1e5
    # the served results equal a direct pooled inversion of each request's queries
    for i in range(0, nreq, 37):
        sl = slice(qoff[i], qoff[i + 1])
        d = [x.cpu().numpy() for x in pool.invert(nurbs.Batch([ids[which[i]]], [0, sizes[i]]),
                                                  torch.as_tensor(P[sl], device="cuda"), 1)]
        assert same_within_tolerance(d, (uv[sl], st[sl], res[sl]), P[sl])
    srv.close()


def test_rejected_requests_and_shutdown(nurbs, served, request):
    """Requests the server cannot take fail with a status (unknown surface and oversized
    request at submission, an invalid surface on its upload ticket); destroying the server with
    requests still queued behind a pause returns promptly (they complete with NURBS_E_STATE)."""
    surfs, pool, ids = served
    srv = nurbs.Server(pool, slots=1, max_batch_queries=256)
    P = queries(surfs[0], 16, np.random.default_rng(8))
    with pytest.raises(nurbs.NurbsError) as e:
        srv.submit_invert(10 ** 6, P)
    assert e.value.code == nurbs.E_INVALID
    with pytest.raises(nurbs.NurbsError) as e:
        srv.submit_invert(int(ids[0]), np.zeros((257, 3)))
    assert e.value.code == nurbs.E_UNSUPPORTED
    bad = dict(surfs[0], knots_u=np.asarray(surfs[0]["knots_u"])[::-1].copy())
    t, sid = srv.submit_upload(bad)
    assert srv.wait(t) == nurbs.E_INVALID and sid[0] < 0
    srv.pause(True)
    for _ in range(3):
        srv.submit_invert(int(ids[0]), P)
    import ctypes as C
    h = srv.h
    srv.h = C.c_void_p()  # destroy through the C-ABI while requests are queued
    assert nurbs.lib().nurbs_server_destroy(h) == 0
