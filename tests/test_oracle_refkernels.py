"""The oracle against the reference itself: the reference's own kernel file
(cuLSH_Kernels.cu) compiled for the host into oracle/_ref and run with the
buffer preparation and launch shapes of its host code (ref_kernels_host.cpp).
Projection epilogue, multiprobe enumeration, the top-K heap and the
distance kernel must agree bit for bit with the oracle. Skipped where the reference tree was not
present at build time (oracle/_ref absent)."""

import numpy as np
import pytest

import oracle
from conftest import golden_cases, load_case

ref = oracle.ref_kernels()
pytestmark = pytest.mark.skipif(ref is None, reason="oracle/_ref not built (no reference tree here)")


def ref_probe_rows(vals, T):
    """vals [M, Q] unfloored -> [Q, T, M] probe codes from the reference kernels."""
    M, Q = vals.shape
    out = np.zeros(M * Q * T, np.float32)
    assert ref.ref_probing_codes(np.ascontiguousarray(vals, np.float32), Q, M, T, out) == 0
    return out.reshape(M, Q, T).transpose(1, 2, 0)


def test_projection_epilogue():
    """fl(fl(C - b) / W) and its floor, C the oracle's FMA chains, for W a
    power of two and not, and values on and near integer boundaries."""
    rng = np.random.default_rng(11)
    for W in (4.0, 16.0, 0.25, 3.0, 6.7, 900.0):
        n, D, L, M = 300, 24, 3, 7
        X = rng.normal(0, 10, (n, D)).astype(np.float32)
        X[:50] = np.round(X[:50])
        A = rng.normal(0, 1, (L, M, D)).astype(np.float32)
        b = rng.uniform(0, W, (L, M)).astype(np.float32)
        b[0, :3] = 0.0
        C = oracle.project(X, A, np.zeros((L, M), np.float32), 1.0)   # the bare chains
        want = oracle.project(X, A, b, W)
        for do_floor in (0, 1):
            got = C.copy()
            assert ref.ref_projection_epilogue(got, n, L * M, b.reshape(-1), W, do_floor) == 0
            expect = np.floor(want) if do_floor else want
            np.testing.assert_array_equal(got, expect, err_msg=f"W={W} floor={do_floor}")


@pytest.mark.parametrize("ties", [False, True])
def test_probe_codes(ties):
    """Every probe row of many queries, M from 1 to 15 and T up to 64, with
    distinct deltas or many exact ties (the heap procedure's order)."""
    rng = np.random.default_rng(12 + ties)
    cases = 0
    for _ in range(150):
        M, T, Q = int(rng.integers(1, 16)), int(rng.integers(1, 65)), int(rng.integers(1, 24))
        if ties:
            vals = (rng.integers(-40, 40, (M, Q)) / 4).astype(np.float32)
        else:
            vals = rng.normal(0, 5, (M, Q)).astype(np.float32)
        got = ref_probe_rows(vals, T)
        for q in range(Q):
            np.testing.assert_array_equal(oracle.probe_one(vals[:, q].copy(), T), got[q],
                                          err_msg=f"M={M} T={T} v={vals[:, q]}")
            cases += 1
    assert cases > 1000


@pytest.mark.parametrize("name", [n for n in golden_cases() if int(load_case(n)["A"].shape[1]) <= 15])
def test_golden_probe_rows(name):
    """The golden cases' own query projections (M <= 15)."""
    c = load_case(name)
    L, M, _ = c["A"].shape
    T = int(c["T"])
    v = oracle.project(c["queries"], c["A"], c["b"], float(c["W"]))
    for l in range(L):
        vals = v[l * M:(l + 1) * M]
        got = ref_probe_rows(vals, T)
        for q in range(vals.shape[1]):
            np.testing.assert_array_equal(oracle.probe_one(vals[:, q].copy(), T), got[q], err_msg=f"table {l} q {q}")


def test_topk_heap():
    """The reference's heap top-K (visit order last candidate first, equal
    distances kept by larger id, output ascending, (-1, FLT_MAX) padding)
    equals the oracle's tie_mode=1, over ragged candidate lists with ties."""
    rng = np.random.default_rng(13)
    cases = 0
    for _ in range(200):
        Q = int(rng.integers(1, 30))
        K = int(rng.choice([1, 2, 3, 5, 10, 17, 33, 100]))
        sizes = rng.integers(0, 60, Q).astype(np.uint32)
        starts = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint32)
        total = int(sizes.sum())
        ids = (np.concatenate([rng.choice(10000, s, replace=False) for s in sizes]) if total
               else np.zeros(0)).astype(np.uint32)
        dist = (rng.integers(0, 20, total) / 2).astype(np.float32)
        oi = np.zeros(Q * K, np.int32)
        od = np.zeros(Q * K, np.float32)
        assert ref.ref_topk(Q, K, ids, starts, sizes, total, dist, oi, od) == 0
        for q in range(Q):
            s, z = int(starts[q]), int(sizes[q])
            wi, wd = oracle.topk(ids[s:s + z], dist[s:s + z], K, tie_mode=1)
            np.testing.assert_array_equal(wi, oi[q * K:(q + 1) * K])
            np.testing.assert_array_equal(wd, od[q * K:(q + 1) * K])
            cases += 1
    assert cases > 1000


def test_distances():
    """The reference's distance kernel (eight lanes, shared-memory tree,
    launched as calculateDistances launches it; its accumulation fused as
    nvcc fuses it) against the oracle's lane-order distance: D from 1 to 299,
    real and integer data, ragged pair counts."""
    rng = np.random.default_rng(14)
    pairs = 0
    for trial in range(40):
        D, N, Q = int(rng.integers(1, 300)), 40, 6
        if trial % 3 == 0:
            data = rng.integers(0, 255, (N, D)).astype(np.float32)
            qs = rng.integers(0, 255, (Q, D)).astype(np.float32)
        else:
            data = rng.normal(0, 3, (N, D)).astype(np.float32)
            qs = rng.normal(0, 3, (Q, D)).astype(np.float32)
        total = int(rng.integers(1, 100))
        cand = rng.integers(0, N, total).astype(np.uint32)
        qidx = rng.integers(0, Q, total).astype(np.uint32)
        out = np.zeros(total, np.float32)
        assert ref.ref_distances(qs, D, Q, data, N, cand, qidx, total, out) == 0
        want = np.array([oracle.distance(qs[qidx[i]], data[cand[i]]) for i in range(total)], np.float32)
        np.testing.assert_array_equal(want, out, err_msg=f"D={D}")
        pairs += total
    assert pairs > 1000


# --- index side: the reference's row sort, bucket boundaries and index file,
# built on Thrust's CPP backend (oracle/_ref/libref_index.so) ---

ref_idx = oracle.ref_index()
needs_ref_index = pytest.mark.skipif(ref_idx is None, reason="oracle/_ref index library not built")


def ref_buckets(P):
    """P: one table's floored codes [M, N] (the reference's N x M column-major)
    -> (ids, starts, sizes) from radixSortRows_1matrix + calculateBuckets."""
    M, N = P.shape
    perm = np.zeros(N, np.uint32)
    starts = np.zeros(N, np.uint32)
    sizes = np.zeros(N, np.uint32)
    nb = np.zeros(1, np.uint32)
    assert ref_idx.ref_sort_buckets(np.ascontiguousarray(P, np.float32), N, M, perm, starts, sizes, nb) == 0
    B = int(nb[0])
    return perm, starts[:B], sizes[:B]


def oracle_buckets(P):
    M, N = P.shape
    ids, starts, sizes = (np.zeros(N, np.uint32) for _ in range(3))
    codes = np.zeros(N * M, np.float32)
    B = oracle.lib().oracle_bucket_table(np.ascontiguousarray(P, np.float32), N, M, ids, starts, sizes, codes)
    return ids, starts[:B], sizes[:B], codes[:B * M].reshape(M, B)


@needs_ref_index
@pytest.mark.parametrize("name", golden_cases())
def test_golden_tables_against_reference_sort(name):
    """Every table of every golden index: the reference's own row sort and
    bucket boundaries, run on the oracle's floored projection, give the
    golden ids, starts and sizes, and the codes the golden file holds are
    the rows those ids point at."""
    c = load_case(name)
    L, M, _ = c["A"].shape
    v = np.floor(oracle.project(c["X"], c["A"], c["b"], float(c["W"])))
    for l in range(L):
        P = v[l * M:(l + 1) * M]
        ids, starts, sizes = ref_buckets(P)
        np.testing.assert_array_equal(ids, c[f"ids_{l}"], err_msg=f"table {l}")
        np.testing.assert_array_equal(starts, c[f"starts_{l}"], err_msg=f"table {l}")
        np.testing.assert_array_equal(sizes, c[f"sizes_{l}"], err_msg=f"table {l}")
        np.testing.assert_array_equal(P[:, ids[starts]], c[f"codes_{l}"], err_msg=f"table {l}")


@needs_ref_index
def test_sort_buckets_random():
    """The oracle's bucket table equals the reference's sort and boundaries
    on random code matrices: N from 1 to 5000, M from 1 to 40, codes drawn
    from a few values (large buckets), a wide range (mostly singletons) or
    mixed signs with zeros, all rows equal, and the values of float32 near
    the integer limits."""
    rng = np.random.default_rng(21)
    cases = 0
    for trial in range(120):
        N, M = int(rng.integers(1, 5000)), int(rng.integers(1, 41))
        kind = trial % 5
        if kind == 0:
            P = rng.integers(-2, 2, (M, N))
        elif kind == 1:
            P = rng.integers(-10**6, 10**6, (M, N))
        elif kind == 2:
            P = rng.integers(-3, 4, (M, N)) * rng.integers(0, 2, (M, N))
        elif kind == 3:
            P = np.full((M, N), float(rng.integers(-5, 5)))
        else:
            P = rng.choice([-2.0**24, -1.0, 0.0, 1.0, 2.0**24, 2.0**31], (M, N))
        P = P.astype(np.float32)
        ids, starts, sizes = ref_buckets(P)
        oids, ostarts, osizes, ocodes = oracle_buckets(P)
        np.testing.assert_array_equal(oids, ids, err_msg=f"N={N} M={M} kind={kind}")
        np.testing.assert_array_equal(ostarts, starts, err_msg=f"N={N} M={M} kind={kind}")
        np.testing.assert_array_equal(osizes, sizes, err_msg=f"N={N} M={M} kind={kind}")
        np.testing.assert_array_equal(ocodes, P[:, ids[starts]], err_msg=f"N={N} M={M} kind={kind}")
        cases += 1
    assert cases == 120


@needs_ref_index
@pytest.mark.parametrize("name", golden_cases())
def test_index_file_through_reference_load_save(name, tmp_path):
    """An index file the oracle writes is read by the reference's
    HashTables::load and written back by its HashTables::save byte for
    byte: the file layout (header, A, b, per-table buckets, ids, starts,
    sizes, codes) is the reference's."""
    c = load_case(name)
    idx = oracle.build_index(c["X"], c["A"], c["b"], float(c["W"]))
    src, out = tmp_path / "oracle.bin", tmp_path / "reference.bin"
    idx.save(str(src))
    assert ref_idx.ref_load_save(str(src).encode(), str(out).encode()) == 0
    assert src.read_bytes() == out.read_bytes()


@needs_ref_index
def test_golden_index_file_through_reference_load_save(tmp_path):
    """The committed golden index file (odd_d13.index.bin) survives the
    reference's load and save unchanged."""
    import os
    from conftest import GOLDEN
    src = os.path.join(GOLDEN, "odd_d13.index.bin")
    out = tmp_path / "reference.bin"
    assert ref_idx.ref_load_save(src.encode(), str(out).encode()) == 0
    with open(src, "rb") as f:
        assert f.read() == out.read_bytes()
