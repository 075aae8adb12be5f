"""Seeded synthetic surfaces and queries for the benchmark workloads.

The reference publishes no dataset; these generators stand in for it with the shapes, sizes
and value distributions of the workloads the engine is measured on:

  small     bicubic 8x8 net, clamped uniform knots (5 spans/direction), z = 0.2 N(0,1),
            w ~ U[0.5,2]; queries S(u,v) + N(0,1e-3) n
  large     bicubic 64x64 net, clamped knots with interior gaps U[0.5,1.5] normalised to [0,1],
            z = 0.1 N(0,1) smoothed once by a 5-point stencil (edges replicate), w ~ U[0.5,2];
            queries S(u,v) + |N(0,1e-2)| n
  batched   4096 surfaces, p,q iid from {2,3,5}, net sizes iid U{4..48} per direction (redrawn
            while n < p+1), knots uniform or gapped (coin flip per direction), z = 0.2 N(0,1),
            w ~ U[0.5,2]; per-surface query counts log-uniform in 16..65536; queries as small
  quintic   degree 5x5, 256x256 net, gapped knots, z = sum of 8 Fourier modes of amplitude 0.05
            with integer frequencies in 1..4, w ~ U[0.5,2] with 1% of weights set to 0.2 or 5;
            queries as small

Normal deviates come from an explicit Box-Muller transform of the generator's uniform doubles,
so the streams do not depend on a library's normal sampler.  Grid x,y = i/(n-1), j/(n-1).
"""
from __future__ import annotations

import math
import numpy as np

SEED_BASE = 20240614
CONFIG_IDS = {"small": 0, "large": 1, "batched": 2, "quintic": 3, "serving": 4}


class Rng:
    def __init__(self, seed: int):
        self.g = np.random.Generator(np.random.PCG64(seed))

    def uniform(self, n, lo=0.0, hi=1.0):
        return lo + (hi - lo) * self.g.random(n)

    def normal(self, n, sigma=1.0):
        m = (n + 1) // 2
        u1 = 1.0 - self.g.random(m)          # (0,1]
        u2 = self.g.random(m)
        r = np.sqrt(-2.0 * np.log(u1))
        z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])[:n]
        return sigma * z

    def integers(self, lo, hi_incl, n=None):
        return self.g.integers(lo, hi_incl + 1, size=n)


def uniform_knots(p: int, n: int) -> np.ndarray:
    """Clamped uniform knot vector of a degree-p, n-point direction on [0,1]."""
    inner = n - p - 1
    return np.concatenate([np.zeros(p + 1), np.arange(1, inner + 1) / (inner + 1), np.ones(p + 1)])


def gapped_knots(p: int, n: int, rng: Rng) -> np.ndarray:
    """Clamped knots whose interior gaps are U[0.5,1.5], normalised to [0,1]."""
    inner = n - p - 1
    gaps = rng.uniform(inner + 1, 0.5, 1.5)
    c = np.cumsum(gaps)
    interior = c[:-1] / c[-1]
    return np.concatenate([np.zeros(p + 1), interior, np.ones(p + 1)])


def _grid(nu, nv, z):
    x = np.repeat(np.arange(nu) / (nu - 1), nv)
    y = np.tile(np.arange(nv) / (nv - 1), nu)
    return np.stack([x, y, z.reshape(-1)], axis=1)


def smooth5(z: np.ndarray) -> np.ndarray:
    """One 5-point-stencil pass, edges replicated: z' = (c + N + S + E + W) / 5."""
    zp = np.pad(z, 1, mode="edge")
    return (zp[1:-1, 1:-1] + zp[:-2, 1:-1] + zp[2:, 1:-1] + zp[1:-1, :-2] + zp[1:-1, 2:]) / 5.0


def surface_small(seed: int = SEED_BASE + 0) -> dict:
    r = Rng(seed)
    p = q = 3
    nu = nv = 8
    z = r.normal(nu * nv, 0.2)
    w = r.uniform(nu * nv, 0.5, 2.0)
    return dict(p=p, q=q, nu=nu, nv=nv, knots_u=uniform_knots(p, nu), knots_v=uniform_knots(q, nv),
                cps=_grid(nu, nv, z), weights=w)


def surface_large(seed: int = SEED_BASE + 1, n: int = 64) -> dict:
    r = Rng(seed)
    p = q = 3
    nu = nv = n
    ku = gapped_knots(p, nu, r)
    kv = gapped_knots(q, nv, r)
    z = smooth5(r.normal(nu * nv, 0.1).reshape(nu, nv))
    w = r.uniform(nu * nv, 0.5, 2.0)
    return dict(p=p, q=q, nu=nu, nv=nv, knots_u=ku, knots_v=kv, cps=_grid(nu, nv, z), weights=w)


def surface_quintic(seed: int = SEED_BASE + 3, n: int = 256) -> dict:
    r = Rng(seed)
    p = q = 5
    nu = nv = n
    ku = gapped_knots(p, nu, r)
    kv = gapped_knots(q, nv, r)
    a = r.integers(1, 4, 8)
    b = r.integers(1, 4, 8)
    phi = r.uniform(8, 0.0, 2 * math.pi)
    x = np.repeat(np.arange(nu) / (nu - 1), nv)
    y = np.tile(np.arange(nv) / (nv - 1), nu)
    z = np.zeros(nu * nv)
    for k in range(8):
        z += 0.05 * np.sin(2 * math.pi * (a[k] * x + b[k] * y) + phi[k])
    w = r.uniform(nu * nv, 0.5, 2.0)
    extreme = r.uniform(nu * nv) < 0.01
    w[extreme] = np.where(r.uniform(int(extreme.sum())) < 0.5, 0.2, 5.0)
    return dict(p=p, q=q, nu=nu, nv=nv, knots_u=ku, knots_v=kv, cps=np.stack([x, y, z], 1), weights=w,
                modes=dict(a=a, b=b, phi=phi))


def surface_random(r: Rng) -> dict:
    """One surface of the batched workload."""
    p = int(r.g.choice([2, 3, 5]))
    q = int(r.g.choice([2, 3, 5]))

    def size(deg):
        while True:
            n = int(r.integers(4, 48))
            if n >= deg + 1:
                return n

    nu, nv = size(p), size(q)
    ku = uniform_knots(p, nu) if r.uniform(1)[0] < 0.5 else gapped_knots(p, nu, r)
    kv = uniform_knots(q, nv) if r.uniform(1)[0] < 0.5 else gapped_knots(q, nv, r)
    z = r.normal(nu * nv, 0.2)
    w = r.uniform(nu * nv, 0.5, 2.0)
    return dict(p=p, q=q, nu=nu, nv=nv, knots_u=ku, knots_v=kv, cps=_grid(nu, nv, z), weights=w)


def batched_surfaces(count: int = 4096, seed: int = SEED_BASE + 2):
    r = Rng(seed)
    surfs = [surface_random(r) for _ in range(count)]
    nq = np.exp(r.uniform(count, math.log(16), math.log(65536))).astype(np.int64)
    return surfs, nq


def query_params(n: int, seed: int, kind: str = "small"):
    """Uniform (u,v) in [0,1]^2 and normal offsets of the workload kind."""
    r = Rng(seed)
    uv = np.stack([r.uniform(n), r.uniform(n)], 1)
    if kind == "large":
        off = np.abs(r.normal(n, 1e-2))
    else:
        off = r.normal(n, 1e-3)
    return uv, off


def form_queries(S: np.ndarray, Su: np.ndarray, Sv: np.ndarray, off: np.ndarray) -> np.ndarray:
    """P = S + off * unit normal, with S, Su, Sv as (n,3) arrays."""
    nrm = np.cross(Su, Sv)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    return S + off[:, None] * nrm
