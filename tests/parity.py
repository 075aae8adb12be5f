"""Parity criteria between the CUDA library and the oracle, shared by the GPU tests.

Evaluation: per output vector, |x - x_ref| <= 1e-12 * max(|x_ref|, 1).
Inversion, per query, by the oracle's status:
  FOUND_UNIQUE     pass if the GPU found it with |uv - uv_ref|_inf <= 1e-9 and
                   residual <= residual_ref * (1 + 1e-12) + 1e-14 * max(1, |P|_inf), or found a
                   strictly closer point (residual < residual_ref - 1e-12, counted as "closer").
                   The absolute term scales with the coordinates: a residual cannot be resolved
                   below the rounding of S itself (~|S| * 1e-16), and for a point lying on the
                   surface the oracle, which reproduces the generating arithmetic, reports 0;
  FOUND_AMBIGUOUS  pass if the GPU residual is no worse (same bound);
  NO_CANDIDATE     the GPU must report NO_CANDIDATE too (candidate sets are bit-exact);
  NOT_CONVERGED    no requirement (counted).
With the oracle's answers at FP32 resolution, FOUND_UNIQUE queries whose answer changes under
them are UNSTABLE (see classify_inversion).
"""
import numpy as np

EVAL_RTOL = 1e-12
UV_TOL = 1e-9


def eval_errors(ev, ref):
    """Max scaled error per 3-row block; points where the reference is NaN are skipped."""
    nb = ref.shape[0] // 3
    out = []
    for b in range(nb):
        r = ref[3 * b:3 * b + 3]
        x = ev[3 * b:3 * b + 3]
        ok = np.all(np.isfinite(r), axis=0)
        nrm = np.maximum(np.linalg.norm(r[:, ok], axis=0), 1.0)
        err = np.linalg.norm(x[:, ok] - r[:, ok], axis=0) / nrm
        out.append(float(err.max()) if err.size else 0.0)
    return out


def stable_mask(ouv, ost, perturbed):
    """FOUND_UNIQUE queries whose answer the oracle also gives for every perturbed copy of the
    point (oracle.OracleSurface.stability_set), to UV_TOL after carrying it back to P."""
    ouv = np.asarray(ouv).reshape(-1, 2)
    puv, pfound, _ = perturbed
    same = np.all(pfound & (np.abs(puv - ouv[None]).max(2) <= UV_TOL), axis=0)
    return (ost == 0) & same


def classify_inversion(uv, st, res, ouv, ost, ores, P, res_abs=1e-14, perturbed=None):
    """res_abs: absolute residual slack per unit of max(1, |P|_inf); 1e-14 unless the surface's
    FP64 evaluation itself is less accurate than that (high degrees), in which case the caller
    passes the measured relative difference of S between the two evaluations.

    perturbed: the oracle's answers at FP32 resolution (OracleSurface.stability_set).  With it,
    FOUND_UNIQUE queries whose answer changes under some of them are UNSTABLE: the oracle itself
    gives different minima for points, or for arithmetic, that FP32 cannot tell apart.  An
    UNSTABLE query passes when the result is found and no farther than the farthest of those
    answers (or when one of them had no answer and none was found); FOUND_UNIQUE queries that are
    stable keep the strict requirement."""
    uv = np.asarray(uv).reshape(-1, 2)
    ouv = np.asarray(ouv).reshape(-1, 2)
    scale = np.maximum(np.abs(np.asarray(P).reshape(-1, 3)).max(1), 1.0)
    found = st <= 1
    no_worse = res <= ores * (1 + 1e-12) + res_abs * scale
    same = found & (np.abs(uv - ouv).max(1) <= UV_TOL) & no_worse
    closer = found & (res < ores - 1e-12)
    uniq = ost == 0
    unstable = np.zeros(len(st), bool)
    fail_us = np.zeros(len(st), bool)
    if perturbed is not None:
        unstable = uniq & ~stable_mask(ouv, ost, perturbed)
        _, pfound, pres = perturbed
        worst = np.maximum(ores, np.where(pfound, pres, -np.inf).max(0))
        some_none = ~np.all(pfound, axis=0)
        ok_us = (found & (res <= worst * (1 + 1e-12) + res_abs * scale)) | (some_none & (st == 3))
        fail_us = unstable & ~ok_us
        uniq = uniq & ~unstable
    amb = ost == 1
    nocand = ost == 2
    nconv = ost == 3
    fail_u = uniq & ~(same | closer)
    fail_a = amb & ~(found & no_worse)
    fail_nc = nocand & (st != 2)
    return dict(n=len(st), unique=int(uniq.sum()), same=int((uniq & same).sum()), closer=int((uniq & closer & ~same).sum()),
                fail_unique=int(fail_u.sum()), unstable=int(unstable.sum()),
                unstable_same=int((unstable & same).sum()), fail_unstable=int(fail_us.sum()),
                ambiguous=int(amb.sum()), fail_ambiguous=int(fail_a.sum()),
                no_candidate=int(nocand.sum()), fail_no_candidate=int(fail_nc.sum()),
                oracle_not_converged=int(nconv.sum()), gpu_found_where_oracle_not=int((nconv & found).sum()),
                max_uv_err_same=float(np.abs(uv - ouv).max(1)[uniq & same].max()) if (uniq & same).any() else 0.0,
                p99_uv_err_same=float(np.percentile(np.abs(uv - ouv).max(1)[uniq & same], 99))
                if (uniq & same).any() else 0.0,
                fail_idx=np.nonzero(fail_u | fail_a | fail_nc | fail_us)[0])


# UNSTABLE queries are counted, not excused wholesale: a test fails when more than this fraction
# of its queries is UNSTABLE (the 64x64 workload has ~0.3 %).
MAX_UNSTABLE_FRAC = 0.01


def oracle_parity(o, P, uv, st, res, res_abs=1e-14):
    """Classifies a GPU inversion against the oracle surface `o`, with the oracle's answers at
    FP32 resolution (OracleSurface.stability_set) deciding which FOUND_UNIQUE queries are
    UNSTABLE."""
    ouv, ost, ores, _ = o.invert(P)
    return classify_inversion(uv, st, res, ouv, ost, ores, P, res_abs=res_abs, perturbed=o.stability_set(P))


def project_parity(o, P, uv, st, res, res_abs=1e-14):
    """Classifies a GPU projection against the oracle's (OracleSurface.project), with its K
    perturbed answers deciding which FOUND_UNIQUE queries are UNSTABLE."""
    ouv, ost, ores, _ = o.project(P)
    return classify_inversion(uv, st, res, ouv, ost, ores, P, res_abs=res_abs,
                              perturbed=o.stability_set(P, project=True))


# Mixed precision only: FOUND_UNIQUE queries whose FP32 exploration ends elsewhere than the
# oracle's FP64 trajectories although the oracle's own FP32-resolution variants agree.  Every
# case examined is a trajectory that leaves the domain far (FP32 cannot evaluate the extrapolated
# polynomial there) or ends just outside an edge; measured 2 in 65,536 queries of the 64x64
# workload and 1 in 16,384 of the quintic one.  The FP64 schedule has none.
MIXED_CHAOS_FRAC = 1e-4


def assert_exact(c, what="", precision=0):
    """No failure in any class (for the mixed schedule, FOUND_UNIQUE failures within
    MIXED_CHAOS_FRAC), and UNSTABLE queries within MAX_UNSTABLE_FRAC."""
    allowed = int(np.ceil(MIXED_CHAOS_FRAC * c["n"])) if precision == 1 else 0
    assert c["fail_unique"] <= allowed, (what, c)
    fails = {k: c[k] for k in ("fail_unstable", "fail_ambiguous", "fail_no_candidate")}
    assert not any(fails.values()), (what, c)
    assert c["unstable"] <= MAX_UNSTABLE_FRAC * c["n"], (what, c)
