"""Generates tests/golden/eval_truth.npz: high-degree surfaces with S..Svv evaluated in 40-digit
arithmetic (mpmath), the yardstick for FP64 evaluation where the span matrices' power basis is
ill-conditioned (degrees 5 and 7).  There, neither the reference's FP64 formulation nor this
library's Horner contraction meets a fixed 1e-12 relative bar; the tests instead require this
library's error against these values to be no larger than the reference's own (the oracle's).

    python tests/golden/make_eval_truth.py      # needs mpmath (not needed to run the tests)

The truth is the rational surface itself: Cox-de Boor basis derivatives (The NURBS Book,
algorithm A2.3) at the FP64 parameters, the homogeneous sums and the quotient rule, all at 40
digits, rounded to FP64 at the end.
"""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEGREES = [(5, 5), (7, 7), (7, 3), (2, 5)]
NPTS = 300


def surface(p, q, nu, nv, seed):
    rng = np.random.default_rng(seed)
    inner = nu - p - 1
    c = np.cumsum(rng.uniform(0.5, 1.5, inner + 1))
    ku = np.concatenate([np.zeros(p + 1), c[:-1] / c[-1], np.ones(p + 1)])
    inner = nv - q - 1
    kv = np.concatenate([np.zeros(q + 1), np.arange(1, inner + 1) / (inner + 1), np.ones(q + 1)])
    x = np.repeat(np.arange(nu) / (nu - 1), nv)
    y = np.tile(np.arange(nv) / (nv - 1), nu)
    z = 0.15 * np.sin(3 * x + 2 * y) + 0.05 * rng.normal(0, 1, nu * nv)
    return dict(p=p, q=q, nu=nu, nv=nv, knots_u=ku, knots_v=kv, cps=np.stack([x, y, z], 1),
                weights=rng.uniform(0.5, 2.0, nu * nv))


def find_span(p, n, U, u):
    """Clamped span as the reference's findSpan computes it."""
    if u >= U[n + 1]:
        return n
    if u <= U[p]:
        return p
    lo, hi = p, n + 1
    mid = (lo + hi) // 2
    while u < U[mid] or u >= U[mid + 1]:
        if u < U[mid]:
            hi = mid
        else:
            lo = mid
        mid = (lo + hi) // 2
    return mid


def basis_ders(mp, i, u, p, U, nd):
    """Derivatives 0..nd of the p+1 non-zero basis functions at u (A2.3)."""
    ndu = [[mp.mpf(0)] * (p + 1) for _ in range(p + 1)]
    ndu[0][0] = mp.mpf(1)
    left = [mp.mpf(0)] * (p + 1)
    right = [mp.mpf(0)] * (p + 1)
    for j in range(1, p + 1):
        left[j] = u - U[i + 1 - j]
        right[j] = U[i + j] - u
        saved = mp.mpf(0)
        for r in range(j):
            ndu[j][r] = right[r + 1] + left[j - r]
            temp = ndu[r][j - 1] / ndu[j][r]
            ndu[r][j] = saved + right[r + 1] * temp
            saved = left[j - r] * temp
        ndu[j][j] = saved
    ders = [[mp.mpf(0)] * (p + 1) for _ in range(nd + 1)]
    for j in range(p + 1):
        ders[0][j] = ndu[j][p]
    a = [[mp.mpf(0)] * (p + 1) for _ in range(2)]
    for r in range(p + 1):
        s1, s2 = 0, 1
        a[0][0] = mp.mpf(1)
        for k in range(1, nd + 1):
            d = mp.mpf(0)
            rk, pk = r - k, p - k
            if r >= k:
                a[s2][0] = a[s1][0] / ndu[pk + 1][rk]
                d = a[s2][0] * ndu[rk][pk]
            j1 = 1 if rk >= -1 else -rk
            j2 = k - 1 if r - 1 <= pk else p - r
            for j in range(j1, j2 + 1):
                a[s2][j] = (a[s1][j] - a[s1][j - 1]) / ndu[pk + 1][rk + j]
                d += a[s2][j] * ndu[rk + j][pk]
            if r <= pk:
                a[s2][k] = -a[s1][k - 1] / ndu[pk + 1][r]
                d += a[s2][k] * ndu[r][pk]
            ders[k][r] = d
            s1, s2 = s2, s1
    f = p
    for k in range(1, nd + 1):
        for j in range(p + 1):
            ders[k][j] *= f
        f *= p - k
    return ders


def truth(mp, sf, uvs):
    p, q, nu, nv = sf["p"], sf["q"], sf["nu"], sf["nv"]
    U = [mp.mpf(float(x)) for x in sf["knots_u"]]
    V = [mp.mpf(float(x)) for x in sf["knots_v"]]
    P = sf["cps"].reshape(nu, nv, 3)
    W = sf["weights"].reshape(nu, nv)
    out = np.zeros((18, len(uvs)))
    for k, (u, v) in enumerate(uvs):
        u, v = mp.mpf(float(u)), mp.mpf(float(v))
        su, sv = find_span(p, nu - 1, U, u), find_span(q, nv - 1, V, v)
        Nu, Nv = basis_ders(mp, su, u, p, U, 2), basis_ders(mp, sv, v, q, V, 2)
        A = {}
        for a in range(3):
            for b in range(3 - a):
                acc = [mp.mpf(0)] * 4
                for i in range(p + 1):
                    for j in range(q + 1):
                        ii, jj = su - p + i, sv - q + j
                        c = Nu[a][i] * Nv[b][j] * mp.mpf(float(W[ii, jj]))
                        for d in range(3):
                            acc[d] += c * mp.mpf(float(P[ii, jj, d]))
                        acc[3] += c
                A[(a, b)] = acc
        w = A[(0, 0)][3]
        S = [A[(0, 0)][d] / w for d in range(3)]
        Su = [(A[(1, 0)][d] - A[(1, 0)][3] * S[d]) / w for d in range(3)]
        Sv = [(A[(0, 1)][d] - A[(0, 1)][3] * S[d]) / w for d in range(3)]
        Suu = [(A[(2, 0)][d] - 2 * A[(1, 0)][3] * Su[d] - A[(2, 0)][3] * S[d]) / w for d in range(3)]
        Suv = [(A[(1, 1)][d] - A[(1, 0)][3] * Sv[d] - A[(0, 1)][3] * Su[d] - A[(1, 1)][3] * S[d]) / w
               for d in range(3)]
        Svv = [(A[(0, 2)][d] - 2 * A[(0, 1)][3] * Sv[d] - A[(0, 2)][3] * S[d]) / w for d in range(3)]
        for bi, blk in enumerate([S, Su, Sv, Suu, Suv, Svv]):
            for d in range(3):
                out[3 * bi + d, k] = float(blk[d])
    return out


def main():
    import mpmath as mp
    mp.mp.dps = 40
    data = {}
    for p, q in DEGREES:
        sf = surface(p, q, max(p + 1, 9), max(q + 1, 7), 100 + 10 * p + q)
        rng = np.random.default_rng(1)
        uv = rng.random((NPTS, 2))
        uv[:4] = [[0, 0], [1, 1], [0, 1], [1, 0]]
        tag = f"p{p}q{q}_"
        for k, v in sf.items():
            data[tag + k] = np.asarray(v)
        data[tag + "uv"] = uv
        data[tag + "truth"] = truth(mp, sf, uv)
        print(tag, "done", flush=True)
    np.savez_compressed(os.path.join(HERE, "eval_truth.npz"), degrees=np.array(DEGREES), **data)


if __name__ == "__main__":
    main()
