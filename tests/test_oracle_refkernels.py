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
