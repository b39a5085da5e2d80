"""Generates the golden fixtures under tests/golden/ from the CPU oracle.

Each case stores its inputs (dataset, queries, A, b, parameters) and the
oracle's outputs: per-table bucket arrays (totalIndices, startingIndices,
sizes, codes), query buckets, kNN ids / squared distances with ties to the
smaller id, the ids the reference's own heap would return (tie_mode 1) and the
per-query candidate counts. One case also carries the index file written in
the reference's save() layout (cuLSH_HashTables.cu:395-438).

Data are quantised to multiples of 1/16 so that they compress well and stay
exact in float32. Run from the repository root:  python tests/golden/make_golden.py
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402


def q16(x):
    return (np.round(np.asarray(x, np.float64) * 16) / 16).astype(np.float32)


def mixture(rng, n, D, centers=20, spread=8.0, noise=1.0):
    c = rng.normal(0, spread, (centers, D))
    pick = rng.integers(0, centers, n)
    return q16(c[pick] + rng.normal(0, noise, (n, D)))


def near(X, rng, q, noise):
    pick = rng.integers(0, X.shape[0], q)
    return q16(X[pick] + rng.normal(0, noise, (q, X.shape[1])))


def case_inputs(name, rng):
    if name == "mix_d16_t1":
        X = mixture(rng, 2000, 16); Qm = near(X, np.random.default_rng(7), 40, 0.5)
        return X, Qm, dict(L=4, M=4, W=8.0, K=10, T=1)
    if name == "mix_d16_t8":
        X = mixture(rng, 2000, 16); Qm = near(X, np.random.default_rng(8), 40, 0.5)
        return X, Qm, dict(L=4, M=4, W=8.0, K=5, T=8)
    if name == "odd_d13":
        X = mixture(rng, 1500, 13); Qm = near(X, np.random.default_rng(9), 30, 0.3)
        return X, Qm, dict(L=3, M=5, W=6.0, K=7, T=4)
    if name == "int_dups":
        X = rng.integers(0, 4, (1500, 8)).astype(np.float32)
        Qm = np.random.default_rng(10).integers(0, 4, (40, 8)).astype(np.float32)
        return X, Qm, dict(L=4, M=3, W=3.0, K=10, T=5)
    if name == "probe_m1":
        X = mixture(rng, 800, 4, spread=3.0); Qm = mixture(np.random.default_rng(11), 25, 4, spread=3.0)
        return X, Qm, dict(L=2, M=1, W=2.0, K=4, T=6)
    if name == "m20_t40":
        X = mixture(rng, 1500, 24); Qm = near(X, np.random.default_rng(12), 20, 0.3)
        return X, Qm, dict(L=2, M=20, W=30.0, K=10, T=40)
    if name == "m40_t70":
        X = mixture(rng, 1000, 16); Qm = near(X, np.random.default_rng(13), 10, 0.3)
        return X, Qm, dict(L=1, M=40, W=40.0, K=10, T=70)
    if name == "heavy":
        base = q16(rng.normal(0, 2, (1, 16)))
        X = np.concatenate([np.repeat(base, 4000, 0), mixture(rng, 2000, 16)])
        X = X[rng.permutation(X.shape[0])]
        Qm = np.concatenate([base + q16(rng.normal(0, 0.05, (6, 16))), mixture(np.random.default_rng(14), 6, 16)])
        return X.astype(np.float32), q16(Qm), dict(L=3, M=4, W=4.0, K=20, T=3)
    if name == "k_gt_cand":
        X = mixture(rng, 1200, 8); Qm = near(X, np.random.default_rng(15), 20, 0.2)
        return X, Qm, dict(L=2, M=6, W=3.0, K=50, T=2)
    if name == "single_bucket":
        X = np.repeat(q16(rng.normal(0, 1, (1, 8))), 500, 0)
        Qm = q16(np.repeat(X[:1], 5, 0) + rng.normal(0, 0.01, (5, 8)))
        return X, Qm, dict(L=2, M=3, W=64.0, K=10, T=2)
    raise KeyError(name)


CASES = ["mix_d16_t1", "mix_d16_t8", "odd_d13", "int_dups", "probe_m1", "m20_t40", "m40_t70", "heavy",
         "k_gt_cand", "single_bucket"]
INDEX_FILE_CASE = "odd_d13"


def make(name):
    rng = np.random.default_rng(sum(map(ord, name)) * 7919)
    X, Qm, p = case_inputs(name, rng)
    N, D = X.shape
    L, M = p["L"], p["M"]
    prng = np.random.default_rng(sum(map(ord, name)) + 1)
    A = q16(prng.normal(0, 1, (L, M, D)))
    b = (prng.random((L, M)) * p["W"]).astype(np.float32)
    idx = oracle.build_index(X, A, b, p["W"])
    r0 = oracle.search(idx, X, Qm, p["K"], p["T"], tie_mode=0)
    r1 = oracle.search(idx, X, Qm, p["K"], p["T"], tie_mode=1)
    out = dict(X=X, queries=Qm, A=A, b=b, W=np.float32(p["W"]), K=np.int32(p["K"]), T=np.int32(p["T"]),
               buckets=idx.buckets.copy())
    for l in range(L):
        out[f"ids_{l}"] = idx.ids(l).copy()
        out[f"starts_{l}"] = idx.starts(l).copy()
        out[f"sizes_{l}"] = idx.sizes(l).copy()
        out[f"codes_{l}"] = idx.codes(l).copy()
    out.update(qbuckets=r0["qbuckets"], knn_ids=r0["knn_ids"], knn_dists=r0["knn_dists"],
               knn_ids_refheap=r1["knn_ids"], knn_dists_refheap=r1["knn_dists"],
               nonunique=r0["nonunique"], unique=r0["unique"])
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    if name == INDEX_FILE_CASE:
        idx.save(os.path.join(HERE, f"{name}.index.bin"))
    div = int(np.sum(np.any(r0["knn_ids"] != r1["knn_ids"], axis=1)))
    print(f"{name}: N={N} D={D} L={L} M={M} T={p['T']} K={p['K']} B={idx.buckets.tolist()} "
          f"nonunique={int(r0['nonunique'].sum())} unique={int(r0['unique'].sum())} "
          f"max_nonunique={int(r0['nonunique'].max())} tie-divergent queries={div}")


if __name__ == "__main__":
    for c in (sys.argv[1:] or CASES):
        make(c)
