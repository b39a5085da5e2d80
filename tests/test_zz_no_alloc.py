"""The search entry point that allocates nothing.

Callers that cannot call cudaMalloc (an allocator owned by someone else, or
a request path where allocation is forbidden) use
culsh_search_run_device_noalloc. Its scratch is a fixed __device__ array
inside libculsh, not memory it allocates. This file checks, through the C
ABI, that it returns what culsh_search_run_device returns (ids bit for bit,
distances within the 1e-5 relative tolerance of the other parity tests) on
two calls in a row for every golden case, that device free memory does not
move between calls, that candidate sets larger than its overflow arena are
admitted in rounds (and that one set alone too large for it is refused), and
that it refuses work beyond its fixed scratch or before the index is on the
device. It is collected last so that a failure here cannot hide the others.
"""

import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases, load_case

pytestmark = pytest.mark.gpu

DIST_RTOL = 1e-5


def _device_index(culsh, torch, c):
    L, M, D = c["A"].shape
    X = torch.from_numpy(c["X"]).cuda()
    ht = culsh.HashTables()
    ht.reset(c["X"].shape[0], D, L, M, float(c["W"]), A=c["A"], b=c["b"])
    ht.index_device(X.data_ptr(), torch.cuda.current_stream().cuda_stream)
    return ht, X


def _noalloc(culsh, st, q, Q, ids, d, stream):
    return culsh.lib().culsh_search_run_device_noalloc(st._h, ctypes.c_void_p(q.data_ptr()), Q,
                                                       ctypes.c_void_p(ids.data_ptr()), ctypes.c_void_p(d.data_ptr()),
                                                       ctypes.c_void_p(stream))


def _expected(culsh, torch, c, st, q, stream):
    Q, K = q.shape[0], int(c["K"])
    want_ids = torch.empty((Q, K), dtype=torch.int32, device="cuda")
    want_d = torch.empty((Q, K), dtype=torch.float32, device="cuda")
    st.search_device(q.data_ptr(), Q, want_ids.data_ptr(), want_d.data_ptr(), stream)
    torch.cuda.synchronize()
    return want_ids.cpu().numpy(), want_d.cpu().numpy()


@pytest.mark.parametrize("name", golden_cases())
def test_noalloc_matches_device_search_twice(culsh, name):
    torch = pytest.importorskip("torch")
    c = load_case(name)
    K, T = int(c["K"]), int(c["T"])
    ht, X = _device_index(culsh, torch, c)
    q = torch.from_numpy(c["queries"]).cuda()
    Q = q.shape[0]
    stream = torch.cuda.current_stream().cuda_stream
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    want_ids, want_d = _expected(culsh, torch, c, st, q, stream)
    np.testing.assert_array_equal(want_ids, c["knn_ids"])

    free = []
    for call in range(2):
        ids = torch.full((Q, K), -7, dtype=torch.int32, device="cuda")
        d = torch.full((Q, K), -7.0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        rc = _noalloc(culsh, st, q, Q, ids, d, stream)
        assert rc == 0, culsh.lib().culsh_last_error().decode()
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        np.testing.assert_array_equal(ids.cpu().numpy(), want_ids, err_msg=f"call {call}")
        np.testing.assert_allclose(d.cpu().numpy(), want_d, rtol=DIST_RTOL, atol=0, err_msg=f"call {call}")
        del ids, d
    assert free[2] == free[3], "the second call changed device free memory"


def test_noalloc_admits_large_candidate_sets_in_rounds(culsh, monkeypatch):
    """'heavy' has candidate sets (a bucket of 4,000 duplicates) that need the
    overflow arena. With the arena capped to hold about one such set, the
    queries that do not fit are re-run in further rounds over the same arena;
    with an arena smaller than one set, the call reports CULSH_ERR_CAPACITY."""
    torch = pytest.importorskip("torch")
    c = load_case("heavy")
    K, T = int(c["K"]), int(c["T"])
    ht, X = _device_index(culsh, torch, c)
    q = torch.from_numpy(c["queries"]).cuda()
    Q = q.shape[0]
    stream = torch.cuda.current_stream().cuda_stream
    st = culsh.SearchTables()
    st.reset(ht, K, T)
    want_ids, want_d = _expected(culsh, torch, c, st, q, stream)
    big = int(c["nonunique"].max())
    words_one = 1
    while words_one < 2 * big:
        words_one *= 2
    words_one += big
    assert int((c["nonunique"] > 2048).sum()) >= 3, "the case must give several arena-sized sets"
    ids = torch.zeros((Q, K), dtype=torch.int32, device="cuda")
    d = torch.zeros((Q, K), dtype=torch.float32, device="cuda")
    for _ in range(2):
        monkeypatch.setenv("CULSH_NOALLOC_ARENA_WORDS", str(words_one + 100))
        rc = _noalloc(culsh, st, q, Q, ids, d, stream)
        assert rc == 0, culsh.lib().culsh_last_error().decode()
        torch.cuda.synchronize()
        np.testing.assert_array_equal(ids.cpu().numpy(), want_ids)
        np.testing.assert_allclose(d.cpu().numpy(), want_d, rtol=DIST_RTOL, atol=0)
    monkeypatch.setenv("CULSH_NOALLOC_ARENA_WORDS", "1000")
    rc = _noalloc(culsh, st, q, Q, ids, d, stream)
    assert rc == culsh.ERR_CAPACITY and "overflow arena" in culsh.lib().culsh_last_error().decode()
    monkeypatch.delenv("CULSH_NOALLOC_ARENA_WORDS")
    rc = _noalloc(culsh, st, q, Q, ids, d, stream)
    assert rc == 0, culsh.lib().culsh_last_error().decode()
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ids.cpu().numpy(), want_ids)


def test_noalloc_refuses_beyond_its_scratch_and_off_device_index(culsh):
    torch = pytest.importorskip("torch")
    c = load_case("mix_d16_t8")
    ht, X = _device_index(culsh, torch, c)
    st = culsh.SearchTables()
    st.reset(ht, int(c["K"]), int(c["T"]))
    q = torch.zeros((4, X.shape[1]), dtype=torch.float32, device="cuda")
    ids = torch.zeros((4, int(c["K"])), dtype=torch.int32, device="cuda")
    d = torch.zeros((4, int(c["K"])), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = _noalloc(culsh, st, q, 5_000_000, ids, d, stream)   # rejected before any launch
    assert rc == culsh.ERR_CAPACITY and "static scratch" in culsh.lib().culsh_last_error().decode()
    loaded = culsh.HashTables()
    loaded.load(os.path.join(GOLDEN, "odd_d13.index.bin"))   # host-resident only
    st2 = culsh.SearchTables()
    st2.reset(loaded, 5, 2)
    rc = _noalloc(culsh, st2, q, 4, ids, d, stream)
    assert rc == culsh.ERR_STATE
