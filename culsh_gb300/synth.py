"""Seeded synthetic workloads for the five measurement configurations.

Every array is float32 in the reference's layout: the dataset and queries are
D x N column-major (here ``[N, D]`` row-major, point-contiguous, the same
bytes), ``A[l]`` is D x M column-major (here ``A[l, m, :]`` is column m) and
``b[l]`` has M entries. Seeds: data 1000+c, queries 2000+c, projection 3000+c.

The generators follow the workload descriptions: Gaussian mixtures, integer
valued non-negative features, unit vectors on the sphere, Zipf-weighted
clusters. They stand in for datasets that cannot be downloaded here.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Config:
    name: str
    N: int
    D: int
    L: int
    M: int
    W: float
    Q: int
    K: int
    T: int


CONFIGS = {
    1: Config("gauss-mixture-100k-d128", 100_000, 128, 8, 8, 4.0, 1_000, 10, 1),
    2: Config("int-features-1m-d128", 1_000_000, 128, 16, 12, 16.0, 10_000, 10, 16),
    3: Config("unit-sphere-1m-d960", 1_000_000, 960, 32, 16, 0.25, 10_000, 10, 64),
    4: Config("zipf-clusters-4m-d128", 4_000_000, 128, 20, 10, 6.0, 100_000, 50, 32),
    5: Config("serving-mixture-10m-d96", 10_000_000, 96, 20, 14, 5.0, 4_096, 10, 8),
}


def _normal(rng, shape, scale=1.0, loc=0.0):
    out = rng.standard_normal(shape, dtype=np.float32)
    if scale != 1.0:
        out *= np.float32(scale)
    if loc != 0.0:
        out += np.float32(loc)
    return out


def _mixture(rng, n, centers, noise):
    choice = rng.integers(0, centers.shape[0], size=n)
    out = _normal(rng, (n, centers.shape[1]), noise)
    out += centers[choice]
    return out


def projection(L: int, M: int, D: int, W: float, seed: int):
    """A ~ N(0,1) with A[l, m, :] the m-th column of table l; b ~ U[0, W)."""
    rng = np.random.default_rng(seed)
    A = _normal(rng, (L, M, D))
    b = (rng.random((L, M), dtype=np.float32) * np.float32(W)).astype(np.float32)
    return A, b


def dataset(c: int, n: int | None = None, q: int | None = None, scale_n: float = 1.0):
    """Returns (X [N, D], queries [Q, D], A [L, M, D], b [L, M], cfg).

    ``n`` / ``q`` override the point and query counts (same generator, same
    seeds), so that small parity cases and bounded CPU samples share the
    distribution of the full workload.
    """
    cfg = CONFIGS[c]
    N = int(n if n is not None else cfg.N * scale_n)
    Q = int(q if q is not None else cfg.Q)
    rd = np.random.default_rng(1000 + c)
    rq = np.random.default_rng(2000 + c)
    D = cfg.D
    if c == 1:
        centers = _normal(rd, (100, D), 10.0)
        X = _mixture(rd, N, centers, 1.0)
        Qm = _mixture(rq, Q, centers, 1.0)
    elif c == 2:
        def feats(r, k):
            v = _normal(r, (k, D), 30.0, 20.0)
            np.maximum(v, 0, out=v)
            np.rint(v, out=v)
            np.minimum(v, 255, out=v)
            return v
        X = feats(rd, N)
        Qm = feats(rq, Q)
    elif c == 3:
        centers = _normal(rd, (1000, D))
        centers /= np.linalg.norm(centers, axis=1, keepdims=True)

        def sphere(r, k):
            v = _mixture(r, k, centers, 0.05)
            v /= np.linalg.norm(v, axis=1, keepdims=True)
            return v
        X = sphere(rd, N)
        Qm = sphere(rq, Q)
    elif c == 4:
        k = 10_000
        centers = _normal(rd, (k, D), 8.0)
        w = 1.0 / np.arange(1, k + 1, dtype=np.float64) ** 1.2
        w /= w.sum()

        def zipf(r, cnt):
            choice = r.choice(k, size=cnt, p=w)
            v = _normal(r, (cnt, D))
            v += centers[choice]
            return v
        X = zipf(rd, N)
        Qm = zipf(rq, Q)
    elif c == 5:
        centers = _normal(rd, (5000, D), 10.0)
        X = _mixture(rd, N, centers, 1.0)
        Qm = _mixture(rq, Q, centers, 1.0)
    else:
        raise ValueError(f"unknown config {c}")
    A, b = projection(cfg.L, cfg.M, D, cfg.W, 3000 + c)
    return np.ascontiguousarray(X, np.float32), np.ascontiguousarray(Qm, np.float32), A, b, cfg
