"""Pins the CPU oracle: hand-traced known answers read off the reference code,
agreement with an independent transliteration (refsim.py), and the committed
golden vectors. CPU only."""

from fractions import Fraction

import numpy as np
import pytest

import oracle
import refsim
from conftest import golden_cases, load_case

F32_MAX = np.float32(np.finfo(np.float32).max)


# ---- multiprobe (cuLSH_Kernels.cu:144-289) ---------------------------------

def test_probe_kat_m2():
    # v = (0.3, 0.9): deltas down (0.3, 0.9), up (0.7, 0.1); ascending order
    # 0.1 (dim1 +1), 0.3 (dim0 -1), 0.7 (dim0 +1), 0.9 (dim1 -1). Traced by
    # hand through kernel_calculateProbingCodes' shift/expand steps.
    rows = oracle.probe_one(np.array([0.3, 0.9], np.float32), 5)
    np.testing.assert_array_equal(rows, [[0, 0], [0, 1], [-1, 0], [-1, 1], [1, 0]])


def test_probe_kat_m1_duplicates():
    # M = 1: once the last delta is in use the combination is never removed, so
    # it is emitted again for every remaining probe (duplicate probes).
    rows = oracle.probe_one(np.array([0.25], np.float32), 6)
    np.testing.assert_array_equal(rows[:, 0], [0, -1, 1, 1, 1, 1])


def test_probe_t1_is_floor():
    v = np.array([-1.5, 2.25, 7.0, -0.0], np.float32)
    np.testing.assert_array_equal(oracle.probe_one(v, 1)[0], np.floor(v))


@pytest.mark.parametrize("M,T", [(1, 4), (2, 9), (3, 11), (5, 16), (12, 16), (16, 64), (20, 40), (40, 70),
                                 (64, 100)])
def test_probe_matches_transliteration(M, T):
    rng = np.random.default_rng(M * 1000 + T)
    for _ in range(6):
        v = (rng.normal(0, 3, M)).astype(np.float32)
        if rng.random() < 0.3:   # exact ties between deltas
            v[: M // 2] = np.float32(0.5)
        np.testing.assert_array_equal(oracle.probe_one(v, T), refsim.probing_codes(v, T))


# ---- top-K (cuLSH_Kernels.cu:356-456) ---------------------------------------

def test_topk_kat_reference_tie_keeps_larger_id():
    # Candidates are visited in descending id order with a strict '<': with
    # three equal distances and K = 1 the reference keeps id 5.
    cand = np.array([1, 3, 5], np.uint32)
    dist = np.array([2.0, 2.0, 2.0], np.float32)
    ids, d = oracle.topk(cand, dist, 1, tie_mode=1)
    assert ids.tolist() == [5] and d.tolist() == [2.0]
    ids, d = oracle.topk(cand, dist, 1, tie_mode=0)
    assert ids.tolist() == [1]


def test_topk_kat_reference_mixed_ties():
    # K = 2, ids 2..5 with distances 0, 1, 1, 1: the reference's heap returns
    # ids (2, 4) - neither smaller-id (2, 3) nor larger-id (2, 5) order.
    cand = np.array([2, 3, 4, 5], np.uint32)
    dist = np.array([0.0, 1.0, 1.0, 1.0], np.float32)
    ids, d = oracle.topk(cand, dist, 2, tie_mode=1)
    assert ids.tolist() == [2, 4] and d.tolist() == [0.0, 1.0]
    ids, _ = oracle.topk(cand, dist, 2, tie_mode=0)
    assert ids.tolist() == [2, 3]


def test_topk_padding():
    ids, d = oracle.topk(np.array([7], np.uint32), np.array([3.0], np.float32), 4, tie_mode=0)
    assert ids.tolist() == [7, -1, -1, -1]
    assert d[0] == 3.0 and np.all(d[1:] == F32_MAX)
    ids1, d1 = oracle.topk(np.array([7], np.uint32), np.array([3.0], np.float32), 4, tie_mode=1)
    assert ids1.tolist() == ids.tolist() and np.array_equal(d1, d)


@pytest.mark.parametrize("K", [1, 2, 3, 7, 10, 16, 33])
def test_topk_matches_transliteration(K):
    rng = np.random.default_rng(K)
    for _ in range(20):
        C = int(rng.integers(0, 60))
        cand = np.sort(rng.choice(1000, C, replace=False)).astype(np.uint32)
        dist = rng.integers(0, 6, C).astype(np.float32)   # many exact ties
        ids, d = oracle.topk(cand, dist, K, tie_mode=1)
        rids, rd = refsim.reference_topk(cand, dist, K)
        np.testing.assert_array_equal(ids, rids)
        np.testing.assert_array_equal(d, rd)
        ids0, d0 = oracle.topk(cand, dist, K, tie_mode=0)
        order = sorted(zip(dist.tolist(), cand.tolist()))[:K]
        assert ids0[: len(order)].tolist() == [i for _, i in order]
        assert np.all(ids0[len(order):] == -1)


# ---- arithmetic order --------------------------------------------------------

def _f32_round(x: Fraction) -> np.float32:
    """Correctly rounded (ties-to-even) float32 of an exact rational."""
    f = np.float32(float(x))
    if Fraction(float(f)) == x:
        return f
    lo, hi = (f, np.nextafter(f, np.float32(np.inf))) if Fraction(float(f)) < x else \
        (np.nextafter(f, np.float32(-np.inf)), f)
    dlo, dhi = x - Fraction(float(lo)), Fraction(float(hi)) - x
    if dlo < dhi:
        return lo
    if dhi < dlo:
        return hi
    return lo if (lo.view(np.uint32) & 1) == 0 else hi


def _fma(a, b, c):
    return _f32_round(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def test_projection_is_sequential_fma_chain():
    rng = np.random.default_rng(3)
    D, W = 37, np.float32(0.7)
    x = rng.normal(0, 10, D).astype(np.float32)
    a = rng.normal(0, 1, D).astype(np.float32)
    b = np.float32(0.3)
    acc = np.float32(0)
    for d in range(D):
        acc = _fma(x[d], a[d], acc)
    expect = np.float32(np.float32(acc - b) / W)
    got = oracle.project(x[None, :], a[None, None, :], np.array([[b]], np.float32), W)[0, 0]
    assert got == expect


def test_distance_lane_order():
    rng = np.random.default_rng(4)
    for D in (1, 7, 8, 13, 128):
        q = rng.normal(0, 10, D).astype(np.float32)
        x = rng.normal(0, 10, D).astype(np.float32)
        s = []
        for j in range(8):
            acc = np.float32(0)
            for c in range(j, D, 8):
                diff = np.float32(q[c] - x[c])
                acc = _fma(diff, diff, acc)
            s.append(acc)
        t = [np.float32(s[i] + s[i + 4]) for i in range(4)]
        expect = np.float32(np.float32(t[0] + t[2]) + np.float32(t[1] + t[3]))
        assert oracle.distance(q, x) == expect


def test_bucket_order_is_lexicographic_and_stable():
    rng = np.random.default_rng(5)
    N, M = 3000, 4
    P = rng.integers(-3, 3, (M, N)).astype(np.float32)
    ids = np.zeros(N, np.uint32)
    starts = np.zeros(N, np.uint32)
    sizes = np.zeros(N, np.uint32)
    codes = np.zeros(N * M, np.float32)
    B = oracle.lib().oracle_bucket_table(np.ascontiguousarray(P), N, M, ids, starts, sizes, codes)
    expect = np.lexsort([np.arange(N)] + [P[m] for m in reversed(range(M))])
    np.testing.assert_array_equal(ids, expect)
    rows = P[:, ids].T
    heads = np.concatenate([[True], np.any(rows[1:] != rows[:-1], axis=1)])
    assert B == heads.sum()
    np.testing.assert_array_equal(starts[:B], np.nonzero(heads)[0])
    np.testing.assert_array_equal(codes[: B * M].reshape(M, B), rows[heads].T)


# ---- golden vectors ----------------------------------------------------------

@pytest.mark.parametrize("name", golden_cases())
def test_oracle_reproduces_golden(name):
    c = load_case(name)
    idx = oracle.build_index(c["X"], c["A"], c["b"], float(c["W"]))
    np.testing.assert_array_equal(idx.buckets, c["buckets"])
    for l in range(idx.L):
        np.testing.assert_array_equal(idx.ids(l), c[f"ids_{l}"])
        np.testing.assert_array_equal(idx.starts(l), c[f"starts_{l}"])
        np.testing.assert_array_equal(idx.sizes(l), c[f"sizes_{l}"])
        np.testing.assert_array_equal(idx.codes(l), c[f"codes_{l}"])
    K, T = int(c["K"]), int(c["T"])
    r = oracle.search(idx, c["X"], c["queries"], K, T, tie_mode=0)
    np.testing.assert_array_equal(r["qbuckets"], c["qbuckets"])
    np.testing.assert_array_equal(r["knn_ids"], c["knn_ids"])
    np.testing.assert_array_equal(r["knn_dists"], c["knn_dists"])
    np.testing.assert_array_equal(r["nonunique"], c["nonunique"])
    np.testing.assert_array_equal(r["unique"], c["unique"])
    r1 = oracle.search(idx, c["X"], c["queries"], K, T, tie_mode=1)
    np.testing.assert_array_equal(r1["knn_ids"], c["knn_ids_refheap"])


def test_golden_probe_rows_match_transliteration():
    """The oracle's probe rows inside a golden case equal refsim's."""
    c = load_case("mix_d16_t8")
    L, M = c["A"].shape[:2]
    T = int(c["T"])
    v = oracle.project(c["queries"], c["A"], c["b"], float(c["W"]))
    for q in range(5):
        for l in range(L):
            vq = v[l * M:(l + 1) * M, q]
            np.testing.assert_array_equal(oracle.probe_one(vq, T), refsim.probing_codes(vq, T))
