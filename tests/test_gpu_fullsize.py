"""Full-size parity: the 100k x 128 Gaussian-mixture workload and the
1M x 128 integer-feature workload, index and search compared bit for bit
against the CPU oracle (the latter also at its recall operating point,
W = 825), plus size-independent properties of the index; the
4M x 128 Zipf-cluster and 10M x 96 serving workloads through whole-table,
sampled-point and search comparisons; the D = 960 unit-sphere workload's
shapes at 100,000 points on both projection kernels."""

import functools

import numpy as np
import pytest

import oracle
from culsh_gb300 import synth

pytestmark = pytest.mark.gpu


def index_properties(ht, N, M):
    """Permutation ids, strictly increasing lexicographic bucket codes, sizes
    that tile [0, N) and ascending ids inside every bucket."""
    for l in range(ht.getL()):
        ids = ht.getBuckets_totalIndices(l)
        starts = ht.getBuckets_startingIndices(l)
        sizes = ht.getBuckets_sizes(l)
        codes = ht.getBuckets_codes(l)
        assert np.array_equal(np.sort(ids), np.arange(N, dtype=np.uint32))
        assert starts[0] == 0 and int(sizes.sum()) == N
        assert np.array_equal(starts[1:], (starts[:-1].astype(np.int64) + sizes[:-1]).astype(np.uint32))
        diff = codes[:, 1:] - codes[:, :-1]
        first = np.argmax(diff != 0, axis=0)
        assert np.all(np.any(diff != 0, axis=0)), "duplicate bucket codes"
        assert np.all(diff[first, np.arange(diff.shape[1])] > 0), "codes not lexicographically increasing"
        inside = np.ones(N, bool)
        inside[starts] = False
        assert np.all(ids[1:][inside[1:]] > ids[:-1][inside[1:]]), "ids not ascending inside a bucket"


@pytest.mark.parametrize("config", [1, 2])
def test_full_size_against_oracle(culsh, config):
    X, Qm, A, b, cfg = synth.dataset(config)
    N, D, L, M, W = X.shape[0], cfg.D, cfg.L, cfg.M, cfg.W
    ht = culsh.HashTables()
    ht.reset(N, D, L, M, W, A=A, b=b)
    ht.index(X)
    ref = oracle.build_index(X, A, b, W)
    np.testing.assert_array_equal(ht.getBuckets(), ref.buckets)
    for l in range(L):
        np.testing.assert_array_equal(ht.getBuckets_totalIndices(l), ref.ids(l))
        np.testing.assert_array_equal(ht.getBuckets_startingIndices(l), ref.starts(l))
        np.testing.assert_array_equal(ht.getBuckets_codes(l), ref.codes(l))
    index_properties(ht, N, M)

    # held-out queries as specified, plus queries near dataset points so the
    # candidate / distance / top-K path carries real work
    rng = np.random.default_rng(99)
    near = (X[rng.integers(0, N, 500)] + rng.normal(0, 0.5, (500, D))).astype(np.float32)
    if config == 2:
        near = np.clip(np.rint(near), 0, 255).astype(np.float32)
    queries = np.concatenate([Qm[:2000], near])
    st = culsh.SearchTables()
    for K, T in {(cfg.K, cfg.T), (cfg.K, 1), (100, cfg.T)}:
        st.reset(ht, K, T)
        st.search(queries, dataset=X)
        want = oracle.search(ref, X, queries, K, T)
        np.testing.assert_array_equal(st.getKnnIds(), want["knn_ids"])
        np.testing.assert_allclose(st.getKnnDistances(), want["knn_dists"], rtol=1e-5, atol=0)
        Q = queries.shape[0]
        for l in range(L):
            np.testing.assert_array_equal(st.getQueryBuckets(l), want["qbuckets"][l].reshape(Q, T))
        assert st.getTotalCandidates_unique() == int(want["unique"].sum())
        assert st.getTotalCandidates_nonUnique() == int(want["nonunique"].sum())
    # every near-data query of the mixture workload finds candidates
    if config == 1:
        assert st.getTotalCandidates_unique() > 0


def test_full_size_recall_point(culsh):
    """The headline operating point at full size: the 1M x 128 integer
    features at W = 825 (recall@10 above 0.9), where a held-out query's
    candidates are half the dataset. Its dense queries take the tensor-core
    exact form with bucket rows; ids, distances, query buckets and both
    candidate totals must equal the oracle's for held-out and near-data
    queries."""
    X, Qm, _, _, cfg = synth.dataset(2)
    N, D, L, M, W, K, T = X.shape[0], cfg.D, cfg.L, cfg.M, 825.0, cfg.K, cfg.T
    A, b = synth.projection(L, M, D, W, 3002)
    ht = culsh.HashTables()
    ht.reset(N, D, L, M, W, A=A, b=b)
    ht.index(X)
    ref = oracle.build_index(X, A, b, W)
    np.testing.assert_array_equal(ht.getBuckets(), ref.buckets)
    rng = np.random.default_rng(825)
    near = np.clip(np.rint(X[rng.integers(0, N, 100)] + rng.normal(0, 2.0, (100, D))), 0, 255).astype(np.float32)
    queries = np.concatenate([Qm[:200], near])
    Q = queries.shape[0]
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    st.search(queries, dataset=X)
    want = oracle.search(ref, X, queries, K, T)
    np.testing.assert_array_equal(st.getKnnIds(), want["knn_ids"])
    np.testing.assert_array_equal(st.getKnnDistances(), want["knn_dists"])
    for l in range(L):
        np.testing.assert_array_equal(st.getQueryBuckets(l), want["qbuckets"][l].reshape(Q, T))
    assert st.getTotalCandidates_unique() == int(want["unique"].sum())
    assert st.getTotalCandidates_nonUnique() == int(want["nonunique"].sum())
    pr = st.profile()
    assert pr["knn_queries"] > 0.9 * Q and pr["knn_fallback"] == 0 and pr["bucket_rows"] > 0


def gpu_index_arrays(ht, N, L, M):
    """The index the GPU built, packed as the oracle packs its own."""
    buckets = np.asarray(ht.getBuckets(), np.uint32)
    ids = np.zeros((L, N), np.uint32)
    starts = np.zeros((L, N), np.uint32)
    sizes = np.zeros((L, N), np.uint32)
    codes = np.zeros((L, N * M), np.float32)
    for l in range(L):
        B = int(buckets[l])
        ids[l] = ht.getBuckets_totalIndices(l)
        starts[l, :B] = ht.getBuckets_startingIndices(l)
        sizes[l, :B] = ht.getBuckets_sizes(l)
        codes[l, :B * M] = ht.getBuckets_codes(l).reshape(-1)
    return buckets, ids, starts, sizes, codes


@pytest.mark.parametrize("config", [4, 5])
def test_full_size_large_configs(culsh, config):
    """The 4M x 128 Zipf-cluster workload (heavy-tailed candidate counts:
    work stealing, dense candidates, overflow) and the 10M x 96 serving
    mixture at full size. Two whole tables are compared with the oracle's;
    in every table the bucket of 20,000 sampled points carries the oracle's
    floored projection of that point; every table passes the index
    properties; and 500 queries (300 held out, 200 near data points, which
    find candidates) are
    searched at the workload's K and T, compared bit for bit with the
    oracle's search over the same index."""
    X, Qm, A, b, cfg = synth.dataset(config)
    N, D, L, M, W = X.shape[0], cfg.D, cfg.L, cfg.M, cfg.W
    ht = culsh.HashTables()
    ht.reset(N, D, L, M, W, A=A, b=b)
    ht.index(X)
    index_properties(ht, N, M)
    buckets, ids, starts, sizes, codes = gpu_index_arrays(ht, N, L, M)

    pick = [0, L - 1]
    ref = oracle.build_index(X, A[pick], b[pick], W)
    for j, l in enumerate(pick):
        B = int(buckets[l])
        assert B == int(ref.buckets[j])
        np.testing.assert_array_equal(ids[l], ref.ids(j), err_msg=f"table {l}")
        np.testing.assert_array_equal(starts[l, :B], ref.starts(j), err_msg=f"table {l}")
        np.testing.assert_array_equal(sizes[l, :B], ref.sizes(j), err_msg=f"table {l}")
        np.testing.assert_array_equal(codes[l, :B * M].reshape(M, B), ref.codes(j), err_msg=f"table {l}")
    del ref

    rng = np.random.default_rng(7)
    pts = np.sort(rng.choice(N, 20_000, replace=False))
    P = np.floor(oracle.project(X[pts], A, b, W))
    pos = np.empty(N, np.int64)
    for l in range(L):
        B = int(buckets[l])
        pos[ids[l]] = np.arange(N)
        bucket = np.searchsorted(starts[l, :B], pos[pts], side="right") - 1
        np.testing.assert_array_equal(codes[l, :B * M].reshape(M, B)[:, bucket], P[l * M:(l + 1) * M],
                                      err_msg=f"table {l}")

    idx = oracle.Index(N, D, L, M, W, A, b, buckets, ids, starts, sizes, codes)
    # near-data queries: at the serving workload's W = 5 with M = 14 even a
    # point 0.5 away per coordinate rarely shares a bucket, so those stay closer
    noise = 0.5 if config == 4 else 0.05
    near = (X[rng.integers(0, N, 200)] + rng.normal(0, noise, (200, D))).astype(np.float32)
    queries = np.ascontiguousarray(np.concatenate([Qm[:300], near]))
    Q = queries.shape[0]
    st = culsh.SearchTables()
    runs = [(cfg.K, cfg.T), (cfg.K, 1)] if config == 4 else [(10, 8), (100, 32)]
    for K, T in runs:
        st.reset(ht, K, T)
        st.search(queries, dataset=X)
        want = oracle.search(idx, X, queries, K, T)
        np.testing.assert_array_equal(st.getKnnIds(), want["knn_ids"], err_msg=f"K={K} T={T}")
        np.testing.assert_array_equal(st.getKnnDistances(), want["knn_dists"], err_msg=f"K={K} T={T}")
        for l in range(L):
            np.testing.assert_array_equal(st.getQueryBuckets(l), want["qbuckets"][l].reshape(Q, T))
        assert st.getTotalCandidates_unique() == int(want["unique"].sum())
        assert st.getTotalCandidates_nonUnique() == int(want["nonunique"].sum())
        assert st.getTotalCandidates_unique() > 0


@functools.lru_cache(maxsize=1)
def sphere_case():
    """100,000 unit vectors of the D = 960 workload, its 200 held-out queries
    plus 200 queries a small step from indexed points, and the oracle's index
    and search (built once for both parametrisations)."""
    X, Qm, A, b, cfg = synth.dataset(3, n=100_000, q=200)
    rng = np.random.default_rng(5)
    near = X[rng.integers(0, X.shape[0], 200)] + rng.normal(0, 0.001, (200, cfg.D)).astype(np.float32)
    near /= np.linalg.norm(near, axis=1, keepdims=True)
    queries = np.ascontiguousarray(np.concatenate([Qm, near]).astype(np.float32))
    ref = oracle.build_index(X, A, b, cfg.W)
    want = oracle.search(ref, X, queries, cfg.K, cfg.T)
    return X, A, b, cfg, queries, ref, want


@pytest.mark.parametrize("force_tc", [False, True])
def test_unit_sphere_d960_shapes(culsh, force_tc, monkeypatch):
    """The high-dimensional precision workload's shapes at 100,000 points:
    unit vectors, D = 960, L = 32, M = 16, W = 0.25, T = 64, K = 10. By
    default the index takes the FP32 SIMT projection (the tensor-core bound
    would leave about 14 % of the codes open here); forced onto the tensor
    cores (CULSH_PROJECT_TC) it must produce the same codes, recomputing the
    open ones in the canonical order. Index and search against the oracle."""
    if force_tc:
        monkeypatch.setenv("CULSH_PROJECT_TC", "1")
    X, A, b, cfg, queries, ref, want = sphere_case()
    N, D, L, M, W = X.shape[0], cfg.D, cfg.L, cfg.M, cfg.W
    ht = culsh.HashTables()
    ht.reset(N, D, L, M, W, A=A, b=b)
    ht.index(X)
    p = ht.profile()
    assert p["tensor_cores"] == (1 if force_tc else 0)
    if force_tc:
        assert p["recomputed"] > 0
    np.testing.assert_array_equal(ht.getBuckets(), ref.buckets)
    for l in range(L):
        np.testing.assert_array_equal(ht.getBuckets_totalIndices(l), ref.ids(l), err_msg=f"table {l}")
        np.testing.assert_array_equal(ht.getBuckets_startingIndices(l), ref.starts(l), err_msg=f"table {l}")
        np.testing.assert_array_equal(ht.getBuckets_codes(l), ref.codes(l), err_msg=f"table {l}")
    st = culsh.SearchTables()
    st.reset(ht, cfg.K, cfg.T)
    st.search(queries, dataset=X)
    np.testing.assert_array_equal(st.getKnnIds(), want["knn_ids"])
    np.testing.assert_array_equal(st.getKnnDistances(), want["knn_dists"])
    assert st.getTotalCandidates_unique() == int(want["unique"].sum())
    assert st.getTotalCandidates_unique() > 0
