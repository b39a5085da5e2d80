"""The batched search form: CUDA-graph capture and replay of the whole query
path, every tuning configuration, and the autotuner. Each configuration must
return exactly the oracle's results (ids, distances, query buckets, counts)."""

import itertools

import numpy as np
import pytest

from conftest import load_case
from test_gpu_parity import build_index, check_search

pytestmark = pytest.mark.gpu


def search_host(culsh, ht, c, st=None):
    st = st or culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    st.search(c["queries"], dataset=c["X"])
    return st


def test_graph_captured_then_replayed(culsh):
    c = load_case("mix_d16_t8")
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    modes = []
    for _ in range(3):
        st.search(c["queries"], dataset=c["X"])
        check_search(st, c)
        modes.append(st.profile()["graph_mode"])
    assert modes == [1, 2, 2]
    # fewer queries: a different plan, captured again, then replayed
    st.search(c["queries"][:7], dataset=c["X"])
    assert st.profile()["graph_mode"] == 1
    np.testing.assert_array_equal(st.getKnnIds(), c["knn_ids"][:7])
    st.search(c["queries"][:7], dataset=c["X"])
    assert st.profile()["graph_mode"] == 2
    np.testing.assert_array_equal(st.getKnnIds(), c["knn_ids"][:7])


def test_graph_off_matches(culsh, monkeypatch):
    c = load_case("heavy")
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.set_graphs(False)
    search_host(culsh, ht, c, st)
    check_search(st, c)
    assert st.profile()["graph_mode"] == 0
    st.set_graphs(True)
    monkeypatch.setenv("CULSH_NO_GRAPH", "1")
    search_host(culsh, ht, c, st)
    assert st.profile()["graph_mode"] == 0
    monkeypatch.delenv("CULSH_NO_GRAPH")
    search_host(culsh, ht, c, st)
    check_search(st, c)
    assert st.profile()["graph_mode"] == 1


def test_graph_follows_index_rebuild(culsh):
    """A rebuilt index (other data, other sizes) re-captures the graph."""
    a, b = load_case("odd_d13"), load_case("int_dups")
    st = culsh.SearchTables()
    for c in (a, b, a):
        ht = build_index(culsh, c)
        for _ in range(2):
            search_host(culsh, ht, c, st)
            check_search(st, c)


@pytest.mark.parametrize("name", ["heavy", "m20_t40", "odd_d13"])
def test_every_tuning_configuration(culsh, name):
    c = load_case(name)
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    M = c["A"].shape[1]
    for tile, pch in itertools.product((0, 1, 2, 3, 4), (1, 2, 4)):
        launches = []
        for split in (0, 1, 2):
            st.set_tuning(proj_tile=tile, probe_batch=pch, probe_split=split)
            st.search(c["queries"], dataset=c["X"])
            check_search(st, c)
            launches.append(st.profile()["launches"])
        assert launches[1] == launches[0] + (M <= 16)   # the split form's lookup kernel
        assert launches[2] == launches[0]               # the tail form looks up in the same kernel
    st.set_tuning(proj_tile=0, probe_batch=2, probe_split=0, candidates_mode=0)
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)
    assert st.profile()["candidates_mode"] == 0
    for wt, chunk, bps, bf, sl in itertools.product((64, 128, 256, 512), (64, 1024, 4096), (0, 1), (0, 1),
                                                     (4096, 8192, 16384)):
        st.set_tuning(candidates_mode=1, ws_threads=wt, ws_chunk=chunk, ws_blocks_per_sm=bps, distance_bf16=bf,
                      ws_set_slots=sl, ws_order=(bps + bf + (sl == 8192) + (wt == 128)) % 2)
        st.search(c["queries"], dataset=c["X"])
        check_search(st, c)
        np.testing.assert_array_equal(st.getKnnDistances(), c["knn_dists"])


@pytest.mark.parametrize("name", ["int_dups", "mix_d16_t8", "odd_d13", "heavy", "m40_t70", "single_bucket",
                                  "k_gt_cand"])
def test_bf16_distance_form_is_exact(culsh, name):
    """BF16 candidate distances + certified FP32 rerank return exactly the
    FP32 form's results. Integer data are exact in bf16, so nothing is
    re-read in FP32 there."""
    c = load_case(name)
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    st.set_tuning(candidates_mode=1, distance_bf16=1, dense_tc=0)   # dense queries: SIMT, not tensor cores
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)
    np.testing.assert_array_equal(st.getKnnDistances(), c["knn_dists"])
    pr = st.profile()
    assert pr["candidates_mode"] == 1
    if np.array_equal(c["X"], np.round(c["X"])) and np.abs(c["X"]).max() <= 256:
        assert pr["rechecked"] == 0
    assert pr["rechecked"] <= st.getTotalCandidates_unique()


def test_bf16_form_extreme_magnitudes_and_ties(culsh):
    """Rows with nonzero magnitudes below 2^-100 (whole rows, or a few
    entries of a row) are always re-read in FP32; many exact distance ties
    (duplicated rows, distances that underflow to 0); both forms agree with
    the oracle. (Magnitudes above 2^100 cannot be indexed: their codes leave
    the int32 range.)"""
    import oracle
    rng = np.random.default_rng(3)
    N, D, L, M, W = 3000, 16, 4, 3, 30.0
    X = rng.normal(0, 2, (N, D)).astype(np.float32)
    X[:40] = np.float32(1e-35) * rng.normal(0, 1, (40, D)).astype(np.float32)
    X[40:80, :4] = np.float32(1e-33) * rng.normal(0, 1, (40, 4)).astype(np.float32)
    X[80:400] = X[400:720]                     # duplicated rows: exact ties
    X[720:1000] = np.round(X[720:1000] * 4) / 4  # exact in bf16
    A = rng.normal(0, 1, (L, M, D)).astype(np.float32)
    b = rng.uniform(0, W, (L, M)).astype(np.float32)
    queries = np.concatenate([X[:5] * 3, X[400:420] + 0.01, X[720:730], X[40:45] * 0.5]).astype(np.float32)
    K, T = 12, 4
    ht = culsh.HashTables()
    ht.reset(N, D, L, M, W, A=A, b=b)
    ht.index(X)
    ref = oracle.search(oracle.build_index(X, A, b, W), X, queries, K, T)
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    # the work-stealing forms (dense queries on the SIMT kernels), then the
    # tensor-core path for the dense queries
    for bf, tc in ((0, 0), (1, 0), (0, 1)):
        st.set_tuning(candidates_mode=1, distance_bf16=bf, dense_tc=tc)
        st.search(queries, dataset=X)
        np.testing.assert_array_equal(st.getKnnIds(), ref["knn_ids"])
        np.testing.assert_array_equal(st.getKnnDistances(), ref["knn_dists"])
        if bf:
            assert st.profile()["rechecked"] > 0


def test_tuning_rejects_out_of_range(culsh):
    st = culsh.SearchTables()
    for bad in ({"probe_batch": 3}, {"proj_tile": 5}, {"ws_threads": 96}, {"ws_chunk": 8}, {"candidates_mode": 2},
                {"distance_bf16": 2}, {"ws_set_slots": 5000}, {"probe_split": 3}, {"ws_order": 3}):
        with pytest.raises(culsh.CulshError) as ei:
            st.set_tuning(**bad)
        assert ei.value.code == culsh.ERR_INVALID_ARGUMENT
    t = st.get_tuning()
    assert (t["probe_batch"], t["candidates_mode"], t["ws_threads"]) == (2, 1, 128)


def test_autotune_keeps_results(culsh):
    torch = pytest.importorskip("torch")
    c = load_case("heavy")
    ht = build_index(culsh, c)
    K, T = int(c["K"]), int(c["T"])
    q = torch.from_numpy(c["queries"]).cuda()
    ids = torch.empty((q.shape[0], K), dtype=torch.int32, device="cuda")
    d = torch.empty((q.shape[0], K), dtype=torch.float32, device="cuda")
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    side = torch.cuda.Stream()
    tune = st.autotune(q.data_ptr(), q.shape[0], ids.data_ptr(), d.data_ptr(), side.cuda_stream)
    assert tune["configs_tried"] >= 120 and tune["search_ms"] > 0
    assert tune["ws_set_slots"] in (4096, 8192, 16384)
    assert tune["distance_bf16"] in (0, 1)
    assert tune["probe_batch"] in (1, 2, 4) and tune["ws_threads"] in (64, 128, 256, 512)
    assert tune["probe_split"] in (0, 1, 2) and tune["ws_order"] in (0, 1)
    assert st.get_tuning()["probe_batch"] == tune["probe_batch"]
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ids.cpu().numpy(), c["knn_ids"])
    np.testing.assert_array_equal(d.cpu().numpy(), c["knn_dists"])
    # the tuned object keeps serving identical results through the graph
    for _ in range(2):
        st.search_device(q.data_ptr(), q.shape[0], ids.data_ptr(), d.data_ptr(), side.cuda_stream)
        side.synchronize()
        np.testing.assert_array_equal(ids.cpu().numpy(), c["knn_ids"])
    assert st.profile()["graph_mode"] == 2


def test_wide_rows_shared_memory_opt_in(culsh):
    """D = 900: an item's dynamic shared memory plus the kernel's static
    shared memory passes the 48 KB default in several configurations; each
    runs (opted in as needed, in any order) and matches the oracle."""
    import oracle
    rng = np.random.default_rng(9)
    N, D, L, M, W = 2500, 900, 3, 4, 60.0
    centers = rng.normal(0, 4, (8, D)).astype(np.float32)
    X = (centers[rng.integers(0, 8, N)] + rng.normal(0, 1, (N, D))).astype(np.float32)
    A = rng.normal(0, 1, (L, M, D)).astype(np.float32)
    b = rng.uniform(0, W, (L, M)).astype(np.float32)
    queries = (X[:24] + rng.normal(0, 0.3, (24, D))).astype(np.float32)
    K, T = 10, 4
    ht = culsh.HashTables()
    ht.reset(N, D, L, M, W, A=A, b=b)
    ht.index(X)
    ref = oracle.search(oracle.build_index(X, A, b, W), X, queries, K, T)
    assert int(ref["unique"].max()) > 0
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    for sl, bf, wt in itertools.product((8192, 4096), (1, 0), (256, 64, 128)):
        st.set_tuning(candidates_mode=1, ws_set_slots=sl, distance_bf16=bf, ws_threads=wt)
        st.search(queries, dataset=X)
        np.testing.assert_array_equal(st.getKnnIds(), ref["knn_ids"])
        np.testing.assert_array_equal(st.getKnnDistances(), ref["knn_dists"])


@pytest.mark.parametrize("name", ["mix_d16_t8", "heavy", "odd_d13"])
def test_host_search_direct_and_copy_paths(culsh, name, monkeypatch):
    """The host search reads 16-byte-aligned queries directly from host memory
    (where the device has pageable memory access) and otherwise stages them;
    an unaligned query buffer always stages. All give the oracle's results."""
    c = load_case(name)
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    D = c["queries"].shape[1]
    buf = np.zeros(c["queries"].size + 1, np.float32)
    unaligned = buf[1:].reshape(c["queries"].shape)   # 4-byte offset from a 16-byte boundary
    unaligned[...] = c["queries"]
    assert unaligned.ctypes.data % 16 == 4
    for env in (None, "1"):
        if env:
            monkeypatch.setenv("CULSH_NO_DIRECT_HOST", env)
        for q in (c["queries"], unaligned):
            st.search(q, dataset=c["X"])
            check_search(st, c)
            np.testing.assert_array_equal(st.getKnnDistances(), c["knn_dists"])
            path = st.profile()["host_path"]
            if env is None and q is c["queries"]:
                assert path in (1, 3)   # 3 where the device reads pageable memory (Grace-Blackwell)
            else:
                assert path == 1
    assert D > 0


@pytest.mark.parametrize("name", ["mix_d16_t8", "odd_d13", "m40_t70"])
def test_host_search_fused_copy_over_changing_buffers(culsh, name, monkeypatch):
    """Where the device reads pageable memory, the projection reads the
    caller's rows itself and copies them to the device for the candidate
    stage (L*M <= 192). The cached search graph is replayed over other host
    buffers by updating its projection node in place: rows in reverse order
    give the rows of results in reverse order, fewer rows capture again. The
    copy-kernel form (CULSH_NO_FUSED_COPY) and direct launches
    (CULSH_NO_GRAPH) give the same results."""
    c = load_case(name)
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    q0 = c["queries"]
    q1 = np.ascontiguousarray(q0[::-1])
    q2 = q0.copy()
    q3 = q0[:7].copy()
    ids, dists = c["knn_ids"], c["knn_dists"]
    want = [(ids, dists), (ids[::-1], dists[::-1]), (ids[:7], dists[:7])]
    seq = [(q0, 0, 1), (q1, 1, 2), (q2, 0, 2), (q1, 1, 2), (q3, 2, 1), (q3, 2, 2), (q0, 0, 1), (q2, 0, 2)]
    for env in (None, "CULSH_NO_FUSED_COPY", "CULSH_NO_GRAPH"):
        monkeypatch.delenv("CULSH_NO_FUSED_COPY", raising=False)
        monkeypatch.delenv("CULSH_NO_GRAPH", raising=False)
        if env:
            monkeypatch.setenv(env, "1")
        for i, (q, w, mode) in enumerate(seq):
            st.search(q, dataset=c["X"])
            np.testing.assert_array_equal(st.getKnnIds(), want[w][0], err_msg=f"{env} step {i}")
            np.testing.assert_array_equal(st.getKnnDistances(), want[w][1], err_msg=f"{env} step {i}")
            p = st.profile()
            if p["host_path"] == 1:
                continue   # no pageable memory access on this device
            assert p["host_path"] == (2 if env == "CULSH_NO_FUSED_COPY" else 3)
            if env == "CULSH_NO_GRAPH":
                assert p["graph_mode"] == 0
            elif env is None and i > 0:
                # replayed (with the node pointed at the new rows) or captured anew
                assert p["graph_mode"] == mode, f"step {i}"


def test_clustered_queries_every_item_shape_and_order(culsh):
    """Clustered data where queries of one cluster share most of their
    candidates (up to ~9,400 non-unique, ~6,300 unique per query): every item
    width, set size with partition size, locality order and distance form
    gives the oracle's ids and distances."""
    import oracle
    rng = np.random.default_rng(2026)
    N, D, L, M, W, Q, K, T = 30000, 32, 4, 4, 24.0, 400, 10, 16
    centers = rng.normal(0, 6, (30, D))
    X = (centers[rng.integers(0, 30, N)] + rng.normal(0, 1, (N, D))).astype(np.float32)
    Qm = (centers[rng.integers(0, 30, Q)] + rng.normal(0, 1, (Q, D))).astype(np.float32)
    A = rng.normal(0, 1, (L, M, D)).astype(np.float32)
    b = rng.uniform(0, W, (L, M)).astype(np.float32)
    ref = oracle.search(oracle.build_index(X, A, b, W), X, Qm, K, T)
    assert int(ref["nonunique"].max()) > 8192
    ht = culsh.HashTables()
    ht.reset(N, D, L, M, W, A=A, b=b)
    ht.index(X)
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    for wt, (sl, ch), order, bf in itertools.product((128, 512), ((4096, 2048), (8192, 4096), (16384, 8192)),
                                                     (0, 1), (0, 1)):
        st.set_tuning(candidates_mode=1, ws_threads=wt, ws_set_slots=sl, ws_chunk=ch, ws_order=order,
                      distance_bf16=bf)
        st.search(Qm, dataset=X)
        np.testing.assert_array_equal(st.getKnnIds(), ref["knn_ids"], err_msg=f"{wt} {sl} {ch} {order} {bf}")
        np.testing.assert_array_equal(st.getKnnDistances(), ref["knn_dists"])
        assert st.getTotalCandidates_unique() == int(ref["unique"].sum())
        assert st.profile()["candidates_mode"] == 1


@pytest.mark.parametrize("graphs", [True, False])
def test_stage_events_off(culsh, graphs):
    """Without stage events the search returns the same results; the profile
    says its stage times were not measured, and the reference-style times are
    zero; with events back on, stage times are measured again."""
    c = load_case("heavy")
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    st.set_graphs(graphs)
    st.set_profiling(False)
    for _ in range(2):
        st.search(c["queries"], dataset=c["X"])
        check_search(st, c)
        np.testing.assert_array_equal(st.getKnnDistances(), c["knn_dists"])
        pr = st.profile()
        assert pr["stage_times"] == 0 and pr["project_ms"] == 0 and pr["candidates_ms"] == 0
        assert pr["launches"] >= 4
        assert st.getTimes()["distances"] == 0
    st.set_profiling(True)
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)
    pr = st.profile()
    assert pr["stage_times"] == 1 and pr["probe_ms"] > 0


def test_wide_items_large_k_and_single_query(culsh):
    """Edge shapes for the wide work-stealing options: a K whose per-warp
    lists cannot fit a 512-thread item beside a 16,384-slot set (the search
    falls back to the per-query kernel), a single query with the locality
    order, and T not a multiple of four in the tail probe form."""
    import oracle
    c = load_case("heavy")
    ht = build_index(culsh, c)
    X, Qm = c["X"], c["queries"]
    L, M, D = c["A"].shape
    idx = oracle.build_index(X, c["A"], c["b"], float(c["W"]))
    st = culsh.SearchTables()
    K, T = 1500, int(c["T"])
    ref = oracle.search(idx, X, Qm, K, T)
    st.reset(ht, K, T)
    st.set_tuning(candidates_mode=1, ws_threads=512, ws_set_slots=16384, ws_chunk=8192, ws_order=1)
    st.search(Qm, dataset=X)
    np.testing.assert_array_equal(st.getKnnIds(), ref["knn_ids"])
    np.testing.assert_array_equal(st.getKnnDistances(), ref["knn_dists"])
    assert st.profile()["candidates_mode"] == 0   # item state too large: per-query kernel
    K = int(c["K"])
    ref1 = oracle.search(idx, X, Qm[:1], K, 7)
    st.reset(ht, K, 7)
    st.set_tuning(ws_threads=512, ws_set_slots=16384, ws_chunk=8192, ws_order=1, probe_split=2)
    st.search(Qm[:1], dataset=X)
    np.testing.assert_array_equal(st.getKnnIds(), ref1["knn_ids"])
    np.testing.assert_array_equal(st.getQueryBuckets(0), ref1["qbuckets"][0].reshape(1, 7))
