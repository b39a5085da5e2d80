"""The index order of multi-word keys: digit passes over the top key word,
then each run of equal top words ordered by its lower words and id (sort form
1), and the passes over every word it falls back to when a run is too long
(form 2, and forced with CULSH_SORT_ALL_WORDS), against the oracle. The data
put points in clusters that share the leading columns' codes exactly and
differ in the trailing columns, with cluster sizes across every run class:
single points, 2 to 8, 9 to 32, 33 to 2,048, and one of 2,049 where asked."""

import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def clustered(sizes, seed):
    """D = 12: dims 0-3 fix the leading six columns (one value per cluster,
    spread so that clusters differ there), dims 4-11 drive the trailing six;
    some points repeat exactly."""
    rng = np.random.default_rng(seed)
    D, L, M, W = 12, 2, 12, 1.0
    A = np.zeros((L, M, D), np.float32)
    A[:, :6, :4] = rng.normal(0, 1, (L, 6, 4))
    A[:, 6:, 4:] = rng.normal(0, 1, (L, 6, 8))
    b = rng.uniform(0, W, (L, M)).astype(np.float32)
    parts = []
    for c, n in enumerate(sizes):
        pts = np.empty((n, D), np.float32)
        pts[:, :4] = rng.normal(0, 30, 4).astype(np.float32)
        pts[:, 4:] = rng.normal(0, 4, (n, 8)).astype(np.float32)
        if n > 3:
            pts[n // 2] = pts[0]          # an exact duplicate inside the run
        parts.append(pts)
    X = np.concatenate(parts)
    X = X[rng.permutation(X.shape[0])]
    return np.ascontiguousarray(X), A, b, W


def check(culsh, X, A, b, W):
    L, M, D = A.shape
    N = X.shape[0]
    ht = culsh.HashTables()
    ht.reset(N, D, L, M, W, A=A, b=b)
    ht.index(X)
    ref = oracle.build_index(X, A, b, W)
    np.testing.assert_array_equal(ht.getBuckets(), ref.buckets)
    for l in range(L):
        np.testing.assert_array_equal(ht.getBuckets_totalIndices(l), ref.ids(l), err_msg=f"table {l}")
        np.testing.assert_array_equal(ht.getBuckets_startingIndices(l), ref.starts(l), err_msg=f"table {l}")
        np.testing.assert_array_equal(ht.getBuckets_sizes(l), ref.sizes(l), err_msg=f"table {l}")
        np.testing.assert_array_equal(ht.getBuckets_codes(l), ref.codes(l), err_msg=f"table {l}")
    return ht.profile()


SIZES = [1] * 800 + [2] * 200 + [3] * 60 + [7] * 40 + [8] * 10 + [9] * 10 + [20] * 6 + [32] * 12 + [33] * 6 + [100] * 6 + [700] * 2 + [2048]


def test_top_word_then_runs(culsh):
    X, A, b, W = clustered(SIZES, 1)
    p = check(culsh, X, A, b, W)
    assert p["key_words"] >= 2
    assert p["sort_form"] == 1


def test_run_too_long_falls_back(culsh):
    X, A, b, W = clustered(SIZES + [2049], 2)
    p = check(culsh, X, A, b, W)
    assert p["key_words"] >= 2
    assert p["sort_form"] == 2


def test_all_words_form_agrees(culsh, monkeypatch):
    X, A, b, W = clustered(SIZES, 3)
    monkeypatch.setenv("CULSH_SORT_ALL_WORDS", "1")
    p = check(culsh, X, A, b, W)
    assert p["sort_form"] == 0
