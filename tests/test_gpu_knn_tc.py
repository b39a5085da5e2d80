"""Tensor-core k-NN path for dense queries (knn_tc.cu) against the oracle.

Queries with at least dense_min non-unique candidates get an N-bit
candidate membership row; tcgen05 GEMM tiles then compute q.x for every point
and the epilogue keeps each query's smallest keys among its candidates. With
CULSH_DENSE_MIN=1 every query with a candidate takes this path, so the golden
cases exercise both forms: the exact form (small-integer data: every sum is an
exact integer) and the bound form (any data: certified lower bounds, exact FP32
lane-order recomputation, exact per-query kernel for what the lists cannot
prove). Ids, distances (bit for bit), query buckets and candidate totals must
equal the oracle's (cuLSH_Kernels.cu:301-348 distances, :356-456 top-K in the
(distance, id) order).
"""

import numpy as np
import pytest

from conftest import golden_cases, load_case
from test_gpu_parity import build_index, check_search

pytestmark = pytest.mark.gpu


@pytest.fixture
def all_dense(monkeypatch):
    monkeypatch.setenv("CULSH_DENSE_MIN", "1")


def _search(culsh, ht, queries, X, K, T, **tuning):
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    if tuning:
        st.set_tuning(**tuning)
    st.search(queries, dataset=X)
    return st


@pytest.mark.parametrize("name", golden_cases())
def test_golden_cases_on_tensor_cores(culsh, name, all_dense):
    c = load_case(name)
    ht = build_index(culsh, c)
    K, T = int(c["K"]), int(c["T"])
    st = _search(culsh, ht, c["queries"], c["X"], K, T, dense_tc=1)
    check_search(st, c)
    np.testing.assert_array_equal(st.getKnnDistances(), c["knn_dists"])
    pr = st.profile()
    assert pr["knn_queries"] == int((c["nonunique"] > 0).sum())
    # the SIMT bitmap kernel serves the same queries identically
    st2 = _search(culsh, ht, c["queries"], c["X"], K, T, dense_tc=0)
    check_search(st2, c)
    assert st2.profile()["knn_queries"] == 0


def _oracle_case(X, queries, A, b, W, K, T):
    import oracle
    idx = oracle.build_index(X, A, b, W)
    return oracle.search(idx, X, queries, K, T)


def _check_against(st, want, Q, X):
    np.testing.assert_array_equal(st.getKnnIds(), want["knn_ids"])
    np.testing.assert_array_equal(st.getKnnDistances(), want["knn_dists"])
    assert st.getTotalCandidates_unique() == int(want["unique"].sum())
    assert st.getTotalCandidates_nonUnique() == int(want["nonunique"].sum())


def test_integer_features_near_exhaustive_exact_form(culsh):
    """The integer-feature generator at a recall-reaching W: candidate sets
    cover about half the dataset, every query takes the exact form."""
    from culsh_gb300 import synth
    X, Qm, _, _, _ = synth.dataset(2, n=40_000, q=300)
    L, M, T, K, W = 16, 12, 16, 10, 825.0
    A, b = synth.projection(L, M, X.shape[1], W, 3002)
    want = _oracle_case(X, Qm, A, b, W, K, T)
    ht = culsh.HashTables()
    ht.reset(X.shape[0], X.shape[1], L, M, W, A=A, b=b)
    ht.index(X)
    st = _search(culsh, ht, Qm, X, K, T, dense_tc=1)
    _check_against(st, want, Qm.shape[0], X)
    pr = st.profile()
    assert pr["knn_queries"] > 0.9 * Qm.shape[0] and pr["knn_fallback"] == 0


def test_gaussian_mixture_bound_form(culsh, all_dense):
    """Real-valued clustered data: the bound form with exact recomputation."""
    from culsh_gb300 import synth
    X, Qm, _, _, _ = synth.dataset(1, n=30_000, q=400)
    L, M, T, K, W = 8, 8, 16, 10, 32.0
    A, b = synth.projection(L, M, X.shape[1], W, 3001)
    want = _oracle_case(X, Qm, A, b, W, K, T)
    ht = culsh.HashTables()
    ht.reset(X.shape[0], X.shape[1], L, M, W, A=A, b=b)
    ht.index(X)
    st = _search(culsh, ht, Qm, X, K, T, dense_tc=1)
    _check_against(st, want, Qm.shape[0], X)
    assert st.profile()["knn_queries"] == int((want["nonunique"] > 0).sum())


@pytest.mark.parametrize("lo,hi", [(-100, 100), (0, 1000), (-3, 3)])
def test_integer_ranges_pick_the_right_form(culsh, all_dense, lo, hi):
    """Small signed integers take the exact form; integers beyond bf16's
    exact range take the bound form; both match the oracle."""
    rng = np.random.default_rng(7 + hi)
    N, D, L, M, T, K = 6000, 24, 4, 5, 6, 10
    X = rng.integers(lo, hi + 1, (N, D)).astype(np.float32)
    Qm = X[rng.integers(0, N, 120)] + rng.integers(-1, 2, (120, D)).astype(np.float32)
    W = float(hi - lo) * 2.0
    A = rng.normal(0, 1, (L, M, D)).astype(np.float32)
    b = (rng.random((L, M)) * W).astype(np.float32)
    want = _oracle_case(X, Qm, A, b, W, K, T)
    ht = culsh.HashTables()
    ht.reset(N, D, L, M, W, A=A, b=b)
    ht.index(X)
    st = _search(culsh, ht, Qm, X, K, T, dense_tc=1)
    _check_against(st, want, Qm.shape[0], X)


def test_bound_form_fallback_on_exact_ties(culsh, all_dense, monkeypatch):
    """Lists of exactly K entries and many points at equal distance: the
    bound cannot prove the K-th place, the query goes to the exact per-query
    kernel, and the result still equals the oracle's."""
    monkeypatch.setenv("CULSH_KNN_LIST_MARGIN", "0")
    rng = np.random.default_rng(11)
    base = rng.normal(0, 5, (300, 16)).astype(np.float32)
    X = np.repeat(base, 20, axis=0) + np.float32(0.25)   # 20 copies of each point
    Qm = base[rng.integers(0, 300, 60)] + rng.normal(0, 0.1, (60, 16)).astype(np.float32)
    L, M, T, K, W = 4, 4, 4, 10, 40.0
    A = rng.normal(0, 1, (L, M, 16)).astype(np.float32)
    b = (rng.random((L, M)) * W).astype(np.float32)
    want = _oracle_case(X, Qm, A, b, W, K, T)
    ht = culsh.HashTables()
    ht.reset(X.shape[0], 16, L, M, W, A=A, b=b)
    ht.index(X)
    st = _search(culsh, ht, Qm, X, K, T, dense_tc=1)
    _check_against(st, want, Qm.shape[0], X)
    assert st.profile()["knn_fallback"] > 0


def test_graph_replay_and_autotune_keep_results(culsh, all_dense):
    torch = pytest.importorskip("torch")
    c = load_case("mix_d16_t8")
    L, M, D = c["A"].shape
    K, T = int(c["K"]), int(c["T"])
    X = torch.from_numpy(c["X"]).cuda()
    q = torch.from_numpy(c["queries"]).cuda()
    ht = culsh.HashTables()
    ht.reset(c["X"].shape[0], D, L, M, float(c["W"]), A=c["A"], b=c["b"])
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    ht.index_device(X.data_ptr(), sp)
    ids = torch.empty((q.shape[0], K), dtype=torch.int32, device="cuda")
    d = torch.empty((q.shape[0], K), dtype=torch.float32, device="cuda")
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    st.set_tuning(dense_tc=1)
    modes = []
    for _ in range(3):
        st.search_device(q.data_ptr(), q.shape[0], ids.data_ptr(), d.data_ptr(), sp)
        stream.synchronize()
        np.testing.assert_array_equal(ids.cpu().numpy(), c["knn_ids"])
        np.testing.assert_array_equal(d.cpu().numpy(), c["knn_dists"])
        modes.append(st.profile()["graph_mode"])
    assert modes[0] == 1 and modes[-1] == 2
    tuned = st.autotune(q.data_ptr(), q.shape[0], ids.data_ptr(), d.data_ptr(), sp)
    assert tuned["dense_tc"] in (0, 1)
    np.testing.assert_array_equal(ids.cpu().numpy(), c["knn_ids"])


@pytest.mark.parametrize("K,T,Q", [(1, 1, 1), (20, 16, 257), (10, 8, 513), (64, 4, 96)])
def test_edge_shapes_exact_form(culsh, all_dense, K, T, Q):
    """Edge shapes of the exact form: N not a multiple of the 128-point tile
    (ragged last tile), Q crossing the 256-query tile (one query alone in its
    tile, or a tile of one), K = 1, T = 1. At K = 64 the per-query lists no
    longer fit shared memory beside the operand rings at D = 128, so the
    dense queries take the SIMT bitmap kernel instead; results are the same."""
    from culsh_gb300 import synth
    X, Qm, _, _, _ = synth.dataset(2, n=5_003, q=Q)
    L, M, W = 6, 8, 600.0
    A, b = synth.projection(L, M, X.shape[1], W, 3002)
    want = _oracle_case(X, Qm, A, b, W, K, T)
    ht = culsh.HashTables()
    ht.reset(X.shape[0], X.shape[1], L, M, W, A=A, b=b)
    ht.index(X)
    st = _search(culsh, ht, Qm, X, K, T, dense_tc=1)
    _check_against(st, want, Q, X)
    pr = st.profile()
    assert pr["knn_queries"] == (int((want["nonunique"] > 0).sum()) if K <= 20 else 0)
    assert pr["knn_fallback"] == 0


@pytest.mark.parametrize("K", [1, 20, 64])
def test_edge_k_bound_form(culsh, all_dense, K):
    """The bound form (real-valued data) at K = 1, 20 and 64 (its lists hold
    K plus a margin; at 64 they do not fit shared memory and the SIMT kernel
    serves the dense queries), N ragged, Q crossing the 128-query tile; K
    above a query's candidate count pads with (-1, FLT_MAX)."""
    from culsh_gb300 import synth
    X, Qm, _, _, _ = synth.dataset(1, n=4_999, q=130)
    L, M, T, W = 6, 6, 8, 40.0
    A, b = synth.projection(L, M, X.shape[1], W, 3001)
    want = _oracle_case(X, Qm, A, b, W, K, T)
    ht = culsh.HashTables()
    ht.reset(X.shape[0], X.shape[1], L, M, W, A=A, b=b)
    ht.index(X)
    st = _search(culsh, ht, Qm, X, K, T, dense_tc=1)
    _check_against(st, want, Qm.shape[0], X)
    assert st.profile()["knn_queries"] == (int((want["nonunique"] > 0).sum()) if K <= 20 else 0)


@pytest.mark.parametrize("W,big_min", [(825.0, None), (825.0, "64"), (825.0, "1"), (825.0, "0"), (600.0, "1")])
def test_bucket_rows(culsh, all_dense, monkeypatch, W, big_min):
    """Membership rows with the index's largest buckets ORed in whole (bucket
    rows) hold the same sets as rows built id by id. Thresholds: the default
    max(1024, N/64) (one bucket here), 64 ids (hundreds of rows), 1 (every
    bucket has a row: a query matches more of them than a block keeps, the
    rest go id by id), none; at W = 600 more buckets than the row cap, so
    only the largest keep rows. Ids, distances and both candidate totals
    equal the oracle's."""
    from culsh_gb300 import synth
    if big_min is not None:
        monkeypatch.setenv("CULSH_BIG_ROWS_MIN", big_min)
    X, Qm, _, _, _ = synth.dataset(2, n=20_000, q=300)
    L, M, T, K = 16, 12, 16, 10
    A, b = synth.projection(L, M, X.shape[1], W, 3002)
    want = _oracle_case(X, Qm, A, b, W, K, T)
    ht = culsh.HashTables()
    ht.reset(X.shape[0], X.shape[1], L, M, W, A=A, b=b)
    ht.index(X)
    st = _search(culsh, ht, Qm, X, K, T, dense_tc=1)
    _check_against(st, want, Qm.shape[0], X)
    pr = st.profile()
    assert pr["knn_queries"] == int((want["nonunique"] > 0).sum())
    if big_min == "0":
        assert pr["bucket_rows"] == 0
    elif big_min == "1" and W == 600.0:
        assert pr["bucket_rows"] == 65535
    else:
        assert pr["bucket_rows"] > 0


def test_bucket_rows_follow_rebuilds_and_loads(culsh, all_dense, monkeypatch, tmp_path):
    """Bucket rows belong to one build of the index: when the same object
    indexes another dataset, and when a saved index is loaded into a new
    object, the rows are made again from the new buckets (stale rows would
    add candidates and change the unique counts)."""
    from culsh_gb300 import synth
    monkeypatch.setenv("CULSH_BIG_ROWS_MIN", "64")
    Xa, Qm, _, _, _ = synth.dataset(2, n=40_000, q=200)
    X1, X2 = np.ascontiguousarray(Xa[:20_000]), np.ascontiguousarray(Xa[20_000:])
    L, M, T, K, W = 16, 12, 16, 10, 825.0
    A, b = synth.projection(L, M, X1.shape[1], W, 3002)
    ht = culsh.HashTables()
    ht.reset(X1.shape[0], X1.shape[1], L, M, W, A=A, b=b)
    want = None
    for X in (X1, X2):
        want = _oracle_case(X, Qm, A, b, W, K, T)
        ht.index(X)
        st = _search(culsh, ht, Qm, X, K, T, dense_tc=1)
        _check_against(st, want, Qm.shape[0], X)
        assert st.profile()["bucket_rows"] > 0
    path = str(tmp_path / "rows.index")
    ht.save(path)
    ht2 = culsh.HashTables()
    ht2.load(path)
    st = _search(culsh, ht2, Qm, X2, K, T, dense_tc=1)
    _check_against(st, want, Qm.shape[0], X2)
    assert st.profile()["bucket_rows"] > 0


def test_bucket_rows_bound_form(culsh, all_dense, monkeypatch):
    """Bucket rows under the bound form (real-valued Gaussian-mixture data):
    certified keys, exact recomputation and the fallback see the same
    membership rows; results equal the oracle's."""
    from culsh_gb300 import synth
    monkeypatch.setenv("CULSH_BIG_ROWS_MIN", "64")
    X, Qm, _, _, _ = synth.dataset(1, n=30_000, q=300)
    L, M, T, K, W = 8, 8, 16, 10, 32.0
    A, b = synth.projection(L, M, X.shape[1], W, 3001)
    want = _oracle_case(X, Qm, A, b, W, K, T)
    ht = culsh.HashTables()
    ht.reset(X.shape[0], X.shape[1], L, M, W, A=A, b=b)
    ht.index(X)
    st = _search(culsh, ht, Qm, X, K, T, dense_tc=1)
    _check_against(st, want, Qm.shape[0], X)
    pr = st.profile()
    assert pr["knn_queries"] == int((want["nonunique"] > 0).sum()) and pr["bucket_rows"] > 0


def test_bucket_rows_graph_replay(culsh, all_dense, monkeypatch):
    """Captured and replayed searches whose membership rows use bucket rows
    return the oracle's results on every replay."""
    torch = pytest.importorskip("torch")
    from culsh_gb300 import synth
    monkeypatch.setenv("CULSH_BIG_ROWS_MIN", "64")
    Xn, Qn, _, _, _ = synth.dataset(2, n=20_000, q=256)
    L, M, T, K, W = 16, 12, 16, 10, 825.0
    A, b = synth.projection(L, M, Xn.shape[1], W, 3002)
    want = _oracle_case(Xn, Qn, A, b, W, K, T)
    X = torch.from_numpy(np.ascontiguousarray(Xn)).cuda()
    q = torch.from_numpy(np.ascontiguousarray(Qn)).cuda()
    ht = culsh.HashTables()
    ht.reset(Xn.shape[0], Xn.shape[1], L, M, W, A=A, b=b)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    ht.index_device(X.data_ptr(), sp)
    ids = torch.empty((q.shape[0], K), dtype=torch.int32, device="cuda")
    d = torch.empty((q.shape[0], K), dtype=torch.float32, device="cuda")
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    st.set_tuning(dense_tc=1)
    modes = []
    for _ in range(3):
        st.search_device(q.data_ptr(), q.shape[0], ids.data_ptr(), d.data_ptr(), sp)
        stream.synchronize()
        np.testing.assert_array_equal(ids.cpu().numpy(), want["knn_ids"])
        np.testing.assert_array_equal(d.cpu().numpy(), want["knn_dists"])
        modes.append(st.profile()["graph_mode"])
        assert st.profile()["bucket_rows"] > 0
    assert modes[0] == 1 and modes[-1] == 2
