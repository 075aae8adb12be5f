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


def classify_inversion(uv, st, res, ouv, ost, ores, P, res_abs=1e-14):
    """res_abs: absolute residual slack per unit of max(1, |P|_inf); 1e-14 unless the surface's
    FP64 evaluation itself is less accurate than that (high degrees), in which case the caller
    passes the measured relative difference of S between the two evaluations."""
    uv = np.asarray(uv).reshape(-1, 2)
    ouv = np.asarray(ouv).reshape(-1, 2)
    scale = np.maximum(np.abs(np.asarray(P).reshape(-1, 3)).max(1), 1.0)
    found = st <= 1
    no_worse = res <= ores * (1 + 1e-12) + res_abs * scale
    same = found & (np.abs(uv - ouv).max(1) <= UV_TOL) & no_worse
    closer = found & (res < ores - 1e-12)
    uniq = ost == 0
    amb = ost == 1
    nocand = ost == 2
    nconv = ost == 3
    fail_u = uniq & ~(same | closer)
    fail_a = amb & ~(found & no_worse)
    fail_nc = nocand & (st != 2)
    return dict(n=len(st), unique=int(uniq.sum()), same=int((uniq & same).sum()), closer=int((uniq & closer & ~same).sum()),
                fail_unique=int(fail_u.sum()), ambiguous=int(amb.sum()), fail_ambiguous=int(fail_a.sum()),
                no_candidate=int(nocand.sum()), fail_no_candidate=int(fail_nc.sum()),
                oracle_not_converged=int(nconv.sum()), gpu_found_where_oracle_not=int((nconv & found).sum()),
                max_uv_err_same=float(np.abs(uv - ouv).max(1)[uniq & same].max()) if (uniq & same).any() else 0.0,
                p99_uv_err_same=float(np.percentile(np.abs(uv - ouv).max(1)[uniq & same], 99))
                if (uniq & same).any() else 0.0,
                fail_idx=np.nonzero(fail_u | fail_a | fail_nc)[0])
