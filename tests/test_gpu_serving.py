"""The serving loop: continuous batching of requests with mixed Q, K, T over
one resident index, concurrent slots, memory admission and latency figures.
Each request's result must be exactly what a lone search of the same queries
returns (bit-identical ids and distances; those are in turn bit-exact against
the oracle by the parity tests)."""

import threading

import numpy as np
import pytest

from conftest import load_case
from test_gpu_parity import build_index

pytestmark = pytest.mark.gpu


def alone(culsh, ht, X, q, K, T):
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    st.search(q, dataset=X)
    return st.getKnnIds(), st.getKnnDistances()


def mixed_requests(c, n, seed):
    rng = np.random.default_rng(seed)
    Qall = c["queries"].shape[0]
    reqs = []
    for _ in range(n):
        lo = int(rng.integers(0, Qall))
        hi = int(rng.integers(lo + 1, Qall + 1))
        K = int(rng.choice([1, 5, 10, 33]))
        T = int(rng.choice([1, 3, 8]))
        reqs.append((c["queries"][lo:hi], K, T))
    return reqs


@pytest.mark.parametrize("name,graphs", [("heavy", False), ("mix_d16_t8", False), ("heavy", True)])
def test_each_result_same_alone_and_in_the_mix(culsh, name, graphs):
    c = load_case(name)
    ht = build_index(culsh, c)
    reqs = mixed_requests(c, 40, seed=5)
    ref = [alone(culsh, ht, c["X"], q, K, T) for q, K, T in reqs]
    with culsh.Server(ht, slots=4, max_batch_queries=64, graphs=graphs) as srv:
        tickets = [srv.submit(q, K, T) for q, K, T in reqs]
        for t, (ids0, d0) in zip(tickets, ref):
            ids, d = srv.wait(t, timeout=120)
            np.testing.assert_array_equal(ids, ids0)
            np.testing.assert_array_equal(d, d0)
        st = srv.stats()
    assert st["requests"] == len(reqs) and st["failed"] == 0
    assert st["queries"] == sum(q.shape[0] for q, _, _ in reqs)
    assert st["batches"] <= len(reqs)
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]


def test_concurrent_submitters_and_overlap(culsh):
    """Requests from several threads at once; batches overlap on the device."""
    c = load_case("heavy")
    ht = build_index(culsh, c)
    reqs = mixed_requests(c, 64, seed=11)
    ref = [alone(culsh, ht, c["X"], q, K, T) for q, K, T in reqs]
    results = [None] * len(reqs)
    with culsh.Server(ht, slots=6, max_batch_queries=16) as srv:
        def client(idx):
            for i in idx:
                q, K, T = reqs[i]
                t = srv.submit(q, K, T)
                results[i] = srv.wait(t, timeout=120)
        threads = [threading.Thread(target=client, args=(range(k, len(reqs), 4),)) for k in range(4)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        st = srv.stats()
    for (ids, d), (ids0, d0) in zip(results, ref):
        np.testing.assert_array_equal(ids, ids0)
        np.testing.assert_array_equal(d, d0)
    assert st["max_in_flight"] >= 2
    assert st["failed"] == 0


def test_memory_admission(culsh):
    """A budget that admits one batch at a time still serves everything; a
    request that alone exceeds the budget fails, the others succeed."""
    c = load_case("mix_d16_t8")
    ht = build_index(culsh, c)
    lib = culsh.lib()
    need_one = lib.culsh_search_estimate_bytes(ht._h, 40, 10, 8)
    assert need_one > 0
    reqs = [(c["queries"][: 1 + i % 40], 10, 8) for i in range(12)]
    ref = [alone(culsh, ht, c["X"], q, K, T) for q, K, T in reqs]
    budget = int(need_one * 1.3) + (40 * 16 * 4 + 40 * 10 * 8)
    with culsh.Server(ht, slots=4, max_batch_queries=40, memory_budget=budget) as srv:
        tickets = [srv.submit(q, K, T) for q, K, T in reqs]
        for t, (ids0, d0) in zip(tickets, ref):
            ids, d = srv.wait(t, timeout=120)
            np.testing.assert_array_equal(ids, ids0)
            np.testing.assert_array_equal(d, d0)
        st = srv.stats()
        assert st["max_in_flight"] == 1
        assert st["peak_device_bytes"] <= budget
        # 600 queries with K = 2048 cannot fit this budget at all
        big = np.repeat(c["queries"], 15, axis=0)
        t_big = srv.submit(big, 2048, 8)
        t_ok = srv.submit(c["queries"][:5], 10, 8)
        with pytest.raises(culsh.CulshError) as ei:
            srv.wait(t_big, timeout=120)
        assert ei.value.code == culsh.ERR_OUT_OF_MEMORY
        ids, _ = srv.wait(t_ok, timeout=120)
        np.testing.assert_array_equal(ids, ref[4][0][:5])


def test_invalid_requests(culsh):
    c = load_case("odd_d13")
    ht = build_index(culsh, c)
    with culsh.Server(ht, slots=1) as srv:
        with pytest.raises(culsh.CulshError) as ei:
            srv.submit(c["queries"][:2], 0, 1)
        assert ei.value.code == culsh.ERR_INVALID_ARGUMENT
        with pytest.raises(culsh.CulshError) as ei:
            srv.submit(c["queries"][:2], 5, 100000)
        assert ei.value.code == culsh.ERR_CAPACITY
        t = srv.submit(c["queries"][:3], int(c["K"]), int(c["T"]))
        ids, _ = srv.wait(t, timeout=60)
        np.testing.assert_array_equal(ids, c["knn_ids"][:3])


def test_server_needs_resident_dataset(culsh, tmp_path):
    c = load_case("odd_d13")
    ht = build_index(culsh, c)
    path = tmp_path / "i.bin"
    ht.save(str(path))
    ht2 = culsh.HashTables()
    ht2.reset(str(path))
    with pytest.raises(culsh.CulshError) as ei:
        culsh.Server(ht2)
    assert ei.value.code == culsh.ERR_STATE


def test_dense_requests_on_tensor_cores(culsh, monkeypatch):
    """Requests whose queries are dense (every query, CULSH_DENSE_MIN=1) run
    the membership rows with bucket rows and the tensor-core k-NN in several
    slots at once; each request's ids and distances equal the oracle's."""
    import oracle
    from culsh_gb300 import synth
    monkeypatch.setenv("CULSH_DENSE_MIN", "1")
    monkeypatch.setenv("CULSH_BIG_ROWS_MIN", "64")
    X, Qm, _, _, _ = synth.dataset(2, n=20_000, q=600)
    L, M, W = 16, 12, 825.0
    A, b = synth.projection(L, M, X.shape[1], W, 3002)
    ht = culsh.HashTables()
    ht.reset(X.shape[0], X.shape[1], L, M, W, A=A, b=b)
    ht.index(X)
    ref_index = oracle.build_index(X, A, b, W)
    rng = np.random.default_rng(23)
    reqs = []
    for _ in range(24):
        lo = int(rng.integers(0, Qm.shape[0] - 1))
        hi = int(min(Qm.shape[0], lo + rng.integers(1, 200)))
        reqs.append((np.ascontiguousarray(Qm[lo:hi]), int(rng.choice([1, 5, 10, 20])), int(rng.choice([1, 8, 16]))))
    with culsh.Server(ht, slots=4, max_batch_queries=256) as srv:
        tickets = [srv.submit(q, K, T) for q, K, T in reqs]
        for t, (q, K, T) in zip(tickets, reqs):
            ids, d = srv.wait(t, timeout=120)
            want = oracle.search(ref_index, X, q, K, T)
            np.testing.assert_array_equal(ids, want["knn_ids"])
            np.testing.assert_array_equal(d, want["knn_dists"])
        st = srv.stats()
    assert st["requests"] == len(reqs) and st["failed"] == 0
