"""Parity of the CUDA path (through the C ABI) against the CPU oracle.

Bucket codes, bucket contents, query buckets and kNN ids are compared bit for
bit; kNN (squared) distances must agree within 1e-5 relative (the kernels
reproduce the reference's lane order, so they are in fact identical, which
test_distances_bit_exact checks separately). Runs on a GB300 only.
"""

import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases, load_case

pytestmark = pytest.mark.gpu

DIST_RTOL = 1e-5


def build_index(culsh, c):
    L, M, D = c["A"].shape
    ht = culsh.HashTables()
    ht.reset(c["X"].shape[0], D, L, M, float(c["W"]), A=c["A"], b=c["b"])
    ht.index(c["X"])
    return ht


def check_index(ht, c):
    L = c["A"].shape[0]
    np.testing.assert_array_equal(ht.getBuckets(), c["buckets"])
    for l in range(L):
        np.testing.assert_array_equal(ht.getBuckets_totalIndices(l), c[f"ids_{l}"], err_msg=f"table {l}")
        np.testing.assert_array_equal(ht.getBuckets_startingIndices(l), c[f"starts_{l}"], err_msg=f"table {l}")
        np.testing.assert_array_equal(ht.getBuckets_sizes(l), c[f"sizes_{l}"], err_msg=f"table {l}")
        np.testing.assert_array_equal(ht.getBuckets_codes(l), c[f"codes_{l}"], err_msg=f"table {l}")


def check_search(st, c):
    L = c["A"].shape[0]
    K, T = int(c["K"]), int(c["T"])
    Q = c["queries"].shape[0]
    np.testing.assert_array_equal(st.getKnnIds(), c["knn_ids"])
    np.testing.assert_allclose(st.getKnnDistances(), c["knn_dists"], rtol=DIST_RTOL, atol=0)
    for l in range(L):
        np.testing.assert_array_equal(st.getQueryBuckets(l), c["qbuckets"][l].reshape(Q, T))
    assert st.getTotalCandidates_unique() == int(c["unique"].sum())
    assert st.getTotalCandidates_nonUnique() == int(c["nonunique"].sum())
    N = c["X"].shape[0]
    assert st.getSelectivity() == pytest.approx(c["unique"].sum() / N / Q, rel=1e-6)
    assert K == st.K


@pytest.mark.parametrize("name", golden_cases())
def test_index_matches_oracle(culsh, name):
    c = load_case(name)
    check_index(build_index(culsh, c), c)


@pytest.mark.parametrize("name", golden_cases())
def test_search_matches_oracle(culsh, name):
    c = load_case(name)
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)


@pytest.mark.parametrize("name", golden_cases())
def test_distances_bit_exact(culsh, name):
    c = load_case(name)
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    st.search(c["queries"], dataset=c["X"])
    np.testing.assert_array_equal(st.getKnnDistances(), c["knn_dists"])


def test_save_matches_oracle_file_bytes(culsh, tmp_path):
    c = load_case("odd_d13")
    ht = build_index(culsh, c)
    out = tmp_path / "gpu.index.bin"
    ht.save(str(out))
    assert out.read_bytes() == open(os.path.join(GOLDEN, "odd_d13.index.bin"), "rb").read()


@pytest.mark.parametrize("name", ["odd_d13", "heavy", "int_dups"])
def test_loaded_index_searches_identically(culsh, name, tmp_path):
    c = load_case(name)
    ht = build_index(culsh, c)
    path = tmp_path / "x.bin"
    ht.save(str(path))
    ht2 = culsh.HashTables()
    ht2.reset(str(path))
    st = culsh.SearchTables()
    st.reset(ht2, int(c["K"]), int(c["T"]))
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)


def test_repeated_search_and_reset(culsh):
    c = load_case("mix_d16_t8")
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    for _ in range(2):
        st.reset(ht, int(c["K"]), int(c["T"]))
        st.search(c["queries"], dataset=c["X"])
        check_search(st, c)
    # a second index() on the same object rebuilds identically
    ht.index(c["X"])
    check_index(ht, c)
    # fewer queries after more: buffers are reused
    st.reset(ht, int(c["K"]), int(c["T"]))
    st.search(c["queries"][:3], dataset=c["X"])
    np.testing.assert_array_equal(st.getKnnIds(), c["knn_ids"][:3])


def test_device_api_matches_host_api(culsh):
    torch = pytest.importorskip("torch")
    c = load_case("int_dups")
    L, M, D = c["A"].shape
    X = torch.from_numpy(c["X"]).cuda()
    q = torch.from_numpy(c["queries"]).cuda()
    K, T = int(c["K"]), int(c["T"])
    ht = culsh.HashTables()
    ht.reset(c["X"].shape[0], D, L, M, float(c["W"]), A=c["A"], b=c["b"])
    stream = torch.cuda.current_stream().cuda_stream
    ht.index_device(X.data_ptr(), stream)
    check_index(ht, c)
    ids = torch.empty((q.shape[0], K), dtype=torch.int32, device="cuda")
    d = torch.empty((q.shape[0], K), dtype=torch.float32, device="cuda")
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    st.search_device(q.data_ptr(), q.shape[0], ids.data_ptr(), d.data_ptr(), stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ids.cpu().numpy(), c["knn_ids"])
    np.testing.assert_array_equal(d.cpu().numpy(), c["knn_dists"])


def test_overflow_arena_and_deferred_admission(culsh, monkeypatch):
    """Candidate sets larger than shared memory use the global arena; with a
    tiny arena the queries are deferred and admitted in chunks; with an arena
    smaller than one query's set the search fails like the reference's
    admission check (cuLSH_SearchTables.cu:303-306). The arena belongs to
    the per-query candidate kernel (the work-stealing kernel partitions
    large sets instead and needs none), so the test selects that kernel."""
    monkeypatch.setenv("CULSH_CANDIDATES_PER_QUERY", "1")
    c = load_case("heavy")
    assert int(c["nonunique"].max()) > 2048
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)
    words_one = 1
    while words_one < 2 * int(c["nonunique"].max()):
        words_one *= 2
    words_one += int(c["nonunique"].max())
    monkeypatch.setenv("CULSH_ARENA_WORDS", str(words_one + 100))   # one large query at a time
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)
    monkeypatch.setenv("CULSH_ARENA_WORDS", "1000")
    with pytest.raises(culsh.CulshError) as ei:
        st.search(c["queries"], dataset=c["X"])
    assert ei.value.code == culsh.ERR_OUT_OF_MEMORY and "Cannot load all candidates" in str(ei.value)
    monkeypatch.delenv("CULSH_ARENA_WORDS")
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)


def test_nonfinite_data_is_rejected(culsh):
    c = load_case("odd_d13")
    X = c["X"].copy()
    X[17, 3] = np.nan
    L, M, D = c["A"].shape
    ht = culsh.HashTables()
    ht.reset(X.shape[0], D, L, M, float(c["W"]), A=c["A"], b=c["b"])
    with pytest.raises(culsh.CulshError) as ei:
        ht.index(X)
    assert ei.value.code == culsh.ERR_NUMERIC


def test_random_projection_reset(culsh):
    ht = culsh.HashTables()
    ht.reset(5000, 32, 3, 7, 2.5, seed=1234)
    A = np.stack([ht.getA(l) for l in range(3)])
    b = np.stack([ht.getb(l) for l in range(3)])
    assert A.shape == (3, 7, 32) and b.shape == (3, 7)
    assert abs(A.mean()) < 0.15 and 0.85 < A.std() < 1.15
    assert np.all(b >= 0) and np.all(b.min(axis=1) == 0) and np.all(b < 2.5)
    ht2 = culsh.HashTables()
    ht2.reset(5000, 32, 3, 7, 2.5, seed=1234)
    np.testing.assert_array_equal(ht2.getA(2), A[2])
    X = np.random.default_rng(0).normal(0, 3, (5000, 32)).astype(np.float32)
    ht.index(X)
    st = culsh.SearchTables()
    st.reset(ht, 5, 3)
    st.search(X[:50], dataset=X)
    ids = st.getKnnIds()
    assert np.all(ids[:, 0] == np.arange(50))     # every query point finds itself first


def test_dropin_cpp_program(culsh, tmp_path):
    """The drop-in C++ header, used exactly like the reference's cuLSH.h."""
    from test_capi_cpu import build_dropin
    c = load_case("int_dups")
    exe = build_dropin(culsh, tmp_path)
    L, M, D = c["A"].shape
    N, Q = c["X"].shape[0], c["queries"].shape[0]
    K, T = int(c["K"]), int(c["T"])
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(np.array([N, D, L, M], np.int32).tobytes())
        f.write(np.float32(c["W"]).tobytes())
        f.write(np.array([Q, K, T], np.int32).tobytes())
        for l in range(L):
            f.write(c["A"][l].tobytes())
        for l in range(L):
            f.write(c["b"][l].tobytes())
        f.write(c["X"].tobytes())
        f.write(c["queries"].tobytes())
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(out, np.uint8)
    ids = raw[: Q * K * 4].view(np.int32).reshape(Q, K)
    d = raw[Q * K * 4: Q * K * 8].view(np.float32).reshape(Q, K)
    np.testing.assert_array_equal(ids, c["knn_ids"])
    np.testing.assert_array_equal(d, c["knn_dists"])
    qb = raw[Q * K * 8: Q * K * 8 + L * Q * T * 4].view(np.int32).reshape(L, Q * T)
    np.testing.assert_array_equal(qb, c["qbuckets"])
    tot = raw[-8:].view(np.uint32)
    assert tot.tolist() == [int(c["unique"].sum()), int(c["nonunique"].sum())]
    oracle_file = tmp_path / "oracle.bin"
    import oracle
    oracle.build_index(c["X"], c["A"], c["b"], float(c["W"])).save(str(oracle_file))
    assert open(str(out) + ".index", "rb").read() == oracle_file.read_bytes()


@pytest.mark.parametrize("name", golden_cases())
def test_search_general_probe_kernel(culsh, name, monkeypatch):
    """The general multiprobe kernel (any M <= 64, T <= 256, keys <= 256 bits)
    gives the same results as the fast path the other tests mostly take."""
    monkeypatch.setenv("CULSH_PROBE_GENERIC", "1")
    c = load_case(name)
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)


@pytest.mark.parametrize("form", ["1", "2"])
@pytest.mark.parametrize("name", golden_cases())
def test_search_split_probe_lookups(culsh, name, form, monkeypatch):
    """Split lookups (every probe enumerated first, then looked up behind the
    key filter: one thread per probe in a second kernel, or the pair's own
    thread at the end of its enumeration) give exactly the fused kernel's
    results: query buckets, non-unique counts, ids and distances."""
    monkeypatch.setenv("CULSH_PROBE_SPLIT", form)
    c = load_case(name)
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)
    np.testing.assert_array_equal(st.getKnnDistances(), c["knn_dists"])


@pytest.mark.parametrize("split", ["0", "1", "2"])
@pytest.mark.parametrize("M,T,ties", [(9, 16, False), (12, 16, False), (12, 16, True), (16, 24, False),
                                       (16, 16, True), (5, 9, True), (10, 32, False), (16, 64, False),
                                       (12, 48, True), (16, 40, True)])
def test_probe_order_register_network(culsh, M, T, ties, split, monkeypatch):
    """For M <= 16 the fast kernel orders the 2M deltas in registers (sorting
    network + merge by counting) and takes the reference's heap procedure
    whenever two deltas tie. Query buckets (the probe order of every table)
    and kNN ids match the oracle. The tie cases mix queries with integer
    projections and W = 4 or 8 (downs are multiples of 1/W, so M > W downs
    must tie, and downs of 1/2 tie with ups) with noisy queries whose deltas
    are all distinct. Every probe form (fused, split, tail lookups) runs. T > 16
    also exercises the capped candidate list of the enumeration."""
    import oracle
    monkeypatch.setenv("CULSH_PROBE_SPLIT", split)
    rng = np.random.default_rng(100 * M + T)
    N, D, L = 3000, 16, 3
    if ties:
        X = rng.integers(-1, 2, (N, D)).astype(np.float32)
        A = rng.integers(-1, 2, (L, M, D)).astype(np.float32)
        b = np.zeros((L, M), np.float32)
        W = 8.0 if M % 2 == 0 else 4.0   # more downs than values k/W: ties in every exact query
        Qm = np.concatenate([X[rng.integers(0, N, 60)],
                             X[rng.integers(0, N, 60)] + rng.normal(0, 0.4, (60, D)).astype(np.float32)])
    else:
        centers = rng.normal(0, 3, (12, D)).astype(np.float32)
        X = centers[rng.integers(0, 12, N)] + rng.normal(0, 0.3, (N, D)).astype(np.float32)
        A = rng.normal(0, 1, (L, M, D)).astype(np.float32)
        W = 4.0
        b = rng.uniform(0, W, (L, M)).astype(np.float32)
        Qm = centers[rng.integers(0, 12, 120)] + rng.normal(0, 0.3, (120, D)).astype(np.float32)
    Qm = np.ascontiguousarray(Qm, np.float32)
    K = 10
    ht = culsh.HashTables()
    ht.reset(N, D, L, M, W, A=A, b=b)
    ht.index(X)
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    st.search(Qm, dataset=X)
    ref = oracle.search(oracle.build_index(X, A, b, W), X, Qm, K, T)
    Q = Qm.shape[0]
    hits = 0
    for l in range(L):
        qb = st.getQueryBuckets(l)
        np.testing.assert_array_equal(qb, ref["qbuckets"][l].reshape(Q, T), err_msg=f"table {l}")
        hits += int((qb[:, 1:] >= 0).sum())
    assert hits > Q   # the comparison covers many non-home probes that found a bucket
    np.testing.assert_array_equal(st.getKnnIds(), ref["knn_ids"])
    np.testing.assert_array_equal(st.getKnnDistances(), ref["knn_dists"])


@pytest.mark.parametrize("name", golden_cases())
def test_index_simt_projection(culsh, name, monkeypatch):
    """The SIMT projection kernel (the form every shape supports) builds the
    same index as the tensor-core kernel most cases take."""
    monkeypatch.setenv("CULSH_PROJECT_SIMT", "1")
    c = load_case(name)
    check_index(build_index(culsh, c), c)


@pytest.mark.parametrize("name", golden_cases())
def test_search_per_query_candidates_kernel(culsh, name, monkeypatch):
    """The per-query candidate kernel (one block per query) and the default
    persistent work-stealing kernel give identical results."""
    monkeypatch.setenv("CULSH_CANDIDATES_PER_QUERY", "1")
    c = load_case(name)
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)
    np.testing.assert_array_equal(st.getKnnDistances(), c["knn_dists"])
    assert st.profile()["candidates_mode"] == 0


def test_work_stealing_partitions_and_overflow_reruns(culsh, monkeypatch):
    """'heavy' splits its larger queries into several id partitions whose
    partial top-K lists are merged; a partition that overflows the shared
    set, or a plan larger than the item buffers, re-runs per query."""
    c = load_case("heavy")
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    st.set_tuning(dense_tc=0)   # every query with candidates in work-stealing partitions
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)
    assert st.profile()["candidates_mode"] == 1
    monkeypatch.setenv("CULSH_WS_PARTITIONS", "1")
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)
    assert st.profile()["candidates_mode"] == 2
    monkeypatch.delenv("CULSH_WS_PARTITIONS")
    monkeypatch.setenv("CULSH_WS_ITEMS", "5")
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)
    assert st.profile()["candidates_mode"] == 2
    monkeypatch.delenv("CULSH_WS_ITEMS")
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)
    assert st.profile()["candidates_mode"] == 1


def test_work_stealing_large_candidate_sets(culsh):
    """Queries with about 90,000 distinct candidates each (64 partitions per
    query) mixed with queries that have none, against the oracle."""
    import oracle
    rng = np.random.default_rng(77)
    N, D, L, M, W = 90000, 8, 3, 2, 40.0
    X = rng.normal(0, 1, (N, D)).astype(np.float32)
    A = rng.normal(0, 1, (L, M, D)).astype(np.float32)
    b = rng.uniform(0, W, (L, M)).astype(np.float32)
    far = np.full((3, D), 500.0, np.float32)
    queries = np.concatenate([X[:5] + 0.01, far, X[5:8]]).astype(np.float32)
    K, T = 16, 3
    ht = culsh.HashTables()
    ht.reset(N, D, L, M, W, A=A, b=b)
    ht.index(X)
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    st.search(queries, dataset=X)
    assert st.profile()["candidates_mode"] == 1
    idx = oracle.build_index(X, A, b, W)
    ref = oracle.search(idx, X, queries, K, T)
    np.testing.assert_array_equal(st.getKnnIds(), ref["knn_ids"])
    np.testing.assert_array_equal(st.getKnnDistances(), ref["knn_dists"])
    assert st.getTotalCandidates_unique() == int(ref["unique"].sum())
    assert st.getTotalCandidates_nonUnique() == int(ref["nonunique"].sum())
    assert int(ref["unique"][:5].min()) > 60000 and int(ref["nonunique"][5:8].max()) == 0
    # 269,900 non-unique candidates per query (>= 32,768): the bitmap kernel
    assert st.profile()["dense_queries"] == 8
    st.set_tuning(distance_bf16=1)
    st.search(queries, dataset=X)
    np.testing.assert_array_equal(st.getKnnIds(), ref["knn_ids"])
    np.testing.assert_array_equal(st.getKnnDistances(), ref["knn_dists"])
    # the bitmap kernel computes FP32 distances; partitions stay for the rest
    assert st.profile()["dense_queries"] == 8
    # dense queries on the SIMT bitmap kernel instead of the tensor cores
    st.set_tuning(distance_bf16=0, dense_tc=0)
    st.search(queries, dataset=X)
    np.testing.assert_array_equal(st.getKnnIds(), ref["knn_ids"])
    np.testing.assert_array_equal(st.getKnnDistances(), ref["knn_dists"])
    assert st.profile()["dense_queries"] == 8 and st.profile()["knn_queries"] == 0


@pytest.mark.parametrize("name", golden_cases())
def test_dense_bitmap_candidates_kernel(culsh, name, monkeypatch):
    """Every query with a candidate routed to the bitmap kernel (threshold
    forced to 1): same ids, distances, buckets and counts as the oracle."""
    monkeypatch.setenv("CULSH_DENSE_MIN", "1")
    c = load_case(name)
    ht = build_index(culsh, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    st.set_tuning(dense_tc=0)   # the SIMT bitmap kernel (test_gpu_knn_tc.py covers the tensor cores)
    st.search(c["queries"], dataset=c["X"])
    check_search(st, c)
    np.testing.assert_array_equal(st.getKnnDistances(), c["knn_dists"])
    assert st.profile()["dense_queries"] == int((c["nonunique"] > 0).sum())


@pytest.mark.parametrize("N,D,L,M,W,integer", [(6000, 700, 4, 10, 30.0, False), (5000, 64, 20, 16, 8.0, False),
                                               (4000, 300, 18, 16, 400.0, True)])
def test_streaming_tensor_core_projection(culsh, N, D, L, M, W, integer, monkeypatch):
    """Projection matrices too large for shared memory (D > 256 or L*M > 256)
    take the streaming tensor-core kernel (K slices of X and A, column
    blocks); every code, bucket and id still matches the oracle. (The
    tensor-core path is forced: for some of these shapes the predicted share
    of codes to recompute would otherwise select the SIMT kernel.)"""
    import oracle
    monkeypatch.setenv("CULSH_PROJECT_TC", "1")
    rng = np.random.default_rng(N + D + L)
    if integer:
        X = np.clip(np.rint(rng.normal(20, 30, (N, D))), 0, 255).astype(np.float32)
    else:
        X = rng.normal(0, 1, (N, D)).astype(np.float32)
    A = rng.normal(0, 1, (L, M, D)).astype(np.float32)
    b = rng.uniform(0, W, (L, M)).astype(np.float32)
    ht = culsh.HashTables()
    ht.reset(N, D, L, M, W, A=A, b=b)
    ht.index(X)
    assert ht.profile()["tensor_cores"] == 1
    ref = oracle.build_index(X, A, b, W)
    np.testing.assert_array_equal(ht.getBuckets(), ref.buckets)
    for l in range(L):
        np.testing.assert_array_equal(ht.getBuckets_codes(l), ref.codes(l), err_msg=f"table {l}")
        np.testing.assert_array_equal(ht.getBuckets_totalIndices(l), ref.ids(l), err_msg=f"table {l}")


def test_cli_index_and_search(culsh, tmp_path):
    """The command-line program (the reference demo's nine arguments) builds
    an index with random projections and searches the first Q points. The
    index it saves matches, byte for byte, the oracle's index built with the
    A and b stored in that file, and its printed selectivity is the oracle's."""
    import re
    import oracle
    from culsh_gb300 import _build
    cli = _build.build_cli()
    rng = np.random.default_rng(77)
    N, D, L, M, W, Q, K, T = 5000, 24, 5, 6, 5.0, 300, 10, 8
    centers = rng.normal(0, 6, (50, D))
    X = (centers[rng.integers(0, 50, N)] + rng.normal(0, 1, (N, D))).astype(np.float32)
    data = tmp_path / "data.bin"
    X.tofile(data)
    saved = tmp_path / "cli.index"
    env = dict(os.environ, CULSH_SAVE_INDEX=str(saved))
    r = subprocess.run([cli, str(data), str(D), str(N), str(L), str(M), str(W), str(Q), str(K), str(T)],
                       capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "seconds to index" in r.stdout and "seconds to search" in r.stdout
    ht = culsh.HashTables()
    ht.reset(str(saved))
    A = np.stack([ht.getA(l) for l in range(L)])
    b = np.stack([ht.getb(l) for l in range(L)])
    ref = oracle.build_index(X, A, b, W)
    ref_file = tmp_path / "oracle.index"
    ref.save(str(ref_file))
    assert saved.read_bytes() == ref_file.read_bytes()
    want = oracle.search(ref, X, X[:Q], K, T)
    sel = float(re.search(r"Selectivity = ([0-9.]+)%", r.stdout).group(1))
    assert sel == pytest.approx(float(want["unique"].sum()) / N / Q, abs=6e-4)
    assert want["unique"].sum() > 0
