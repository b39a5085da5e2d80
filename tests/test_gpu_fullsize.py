"""Full-size parity: the 100k x 128 Gaussian-mixture workload and the
1M x 128 integer-feature workload, index and search compared bit for bit
against the CPU oracle, plus size-independent properties of the index."""

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
