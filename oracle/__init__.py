"""CPU oracle for cuLSH's Euclidean LSH index build and search.

TEST INFRASTRUCTURE ONLY: tests/, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` load this module
as the checker. The product (``culsh_gb300``) never imports it.

The arithmetic lives in ``oracle.cpp`` (a C++17 + OpenMP restatement of the
reference, each function citing ``cuLSH_*.cu`` file:line). This module only
builds it (``make -C oracle``) and wraps it with numpy arrays.

Parity status: the reference ships no tests, fixtures or CPU path, and its
build needs a GPU. The oracle is pinned against the reference's own kernel
file compiled for the host (``make -C oracle ref`` into ``oracle/_ref``, run
by ``ref_kernels()``: projection epilogue, multiprobe enumeration, top-K
heap, distances), against the reference's index-side host code built on
Thrust's CPP backend (``ref_index()``: row sort, bucket boundaries, index
file load/save), against the reference's whole index and search path built
the same way (``ref_pipeline()``), where the reference tree is present, and
by hand-traced known answers
and an independent transliteration (tests/refsim.py).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "liboracle.so")
_REF_PATH = os.path.join(_HERE, "_ref", "libref_kernels.so")
_REF_INDEX_PATH = os.path.join(_HERE, "_ref", "libref_index.so")
_REF_PIPELINE_PATH = os.path.join(_HERE, "_ref", "libref_pipeline.so")
_lock = threading.Lock()
_lib = None
_ref = None
_ref_index = None
_ref_pipeline = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_i64 = ctypes.c_int64
_int = ctypes.c_int
_flt = ctypes.c_float


def build() -> str:
    """Compile the oracle shared library (idempotent)."""
    src = os.path.join(_HERE, "oracle.cpp")
    if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


# Where the reference tree is read from by the `ref` recipe (the only place
# that reads it); CULSH_REFERENCE_TREE overrides it.
REFERENCE_TREE = os.environ.get("CULSH_REFERENCE_TREE", "/root/reference")


def build_ref() -> str | None:
    """Compile the reference's kernel file and its index-side host code for the
    host into oracle/_ref when the reference tree is present (the Makefile's
    `ref` target); returns the kernel library's path, or None when it was not
    built."""
    srcs = [os.path.join(_HERE, f) for f in ("ref_kernels_host.cpp", "ref_shim.h", "ref_index_host.cpp",
                                               "ref_index_shim.h", "ref_pipeline_host.cpp", "ref_pipeline_shim.h",
                                               "Makefile", "oracle.cpp")]
    newest = max(os.path.getmtime(f) for f in srcs)
    outs = (_REF_PATH, _REF_INDEX_PATH, _REF_PIPELINE_PATH)
    if any(not os.path.exists(p) or os.path.getmtime(p) < newest for p in outs):
        subprocess.run(["make", "-s", "-C", _HERE, "ref", f"REF={REFERENCE_TREE}"], check=True)
    return _REF_PATH if os.path.exists(_REF_PATH) else None


def ref_kernels():
    """The reference's own kernels run on the host (oracle/_ref), or None when
    they were not built here (no reference tree) or do not load on this
    machine."""
    global _ref
    with _lock:
        if _ref is None:
            if not os.path.exists(_REF_PATH):
                return None
            try:
                R = ctypes.CDLL(_REF_PATH)
            except OSError:
                return None
            R.ref_projection_epilogue.argtypes = [_f32p, _int, _int, _f32p, _flt, _int]
            R.ref_probing_codes.argtypes = [_f32p, _int, _int, _int, _f32p]
            R.ref_topk.argtypes = [_int, _int, _u32p, _u32p, _u32p, ctypes.c_uint, _f32p, _i32p, _f32p]
            R.ref_distances.argtypes = [_f32p, _int, _int, _f32p, _int, _u32p, _u32p, ctypes.c_uint, _f32p]
            _ref = R
    return _ref


def ref_index():
    """The reference's index-side host code (row sort, bucket boundaries,
    HashTables load/save) built on Thrust's CPP backend (oracle/_ref), or
    None when it was not built here or does not load on this machine."""
    global _ref_index
    with _lock:
        if _ref_index is None:
            if not os.path.exists(_REF_INDEX_PATH):
                return None
            try:
                R = ctypes.CDLL(_REF_INDEX_PATH)
            except OSError:
                return None
            R.ref_sort_buckets.argtypes = [_f32p, _int, _int, _u32p, _u32p, _u32p, _u32p]
            R.ref_load_save.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
            _ref_index = R
    return _ref_index


def ref_pipeline_lib():
    """The reference's whole index and search path built for the host
    (oracle/_ref/libref_pipeline.so: Thrust's CPP backend, its kernels run as
    host loops, the oracle's chain for its one GEMM), or None when it was not
    built here or does not load on this machine."""
    global _ref_pipeline
    with _lock:
        if _ref_pipeline is None:
            if not os.path.exists(_REF_PIPELINE_PATH):
                return None
            try:
                R = ctypes.CDLL(_REF_PIPELINE_PATH)
            except OSError:
                return None
            R.ref_pipeline.argtypes = [_f32p, _int, _int, _int, _int, _flt, _f32p, _f32p, _f32p, _int, _int, _int,
                                       ctypes.c_ulonglong, _u32p, _u32p, _u32p, _u32p, _f32p, _i32p, _i32p, _f32p,
                                       _u32p]
            _ref_pipeline = R
    return _ref_pipeline


def ref_pipeline(X, A, b, W, queries, K, T, free_bytes=0):
    """Index X and search the queries with the reference's own host-built
    code. Returns a dict shaped like search() (plus the index arrays and
    totals), or raises RuntimeError with the stage that failed."""
    R = ref_pipeline_lib()
    if R is None:
        raise RuntimeError("oracle/_ref/libref_pipeline.so is not built")
    X = _c(X, np.float32)
    A = _c(A, np.float32)
    b = _c(b, np.float32)
    queries = _c(queries, np.float32)
    L, M, D = A.shape
    N, Q = X.shape[0], queries.shape[0]
    buckets = np.zeros(L, np.uint32)
    ids = np.zeros((L, N), np.uint32)
    starts = np.zeros((L, N), np.uint32)
    sizes = np.zeros((L, N), np.uint32)
    codes = np.zeros((L, N * M), np.float32)
    qb = np.zeros((L, Q * T), np.int32)
    kid = np.zeros((Q, K), np.int32)
    kd = np.zeros((Q, K), np.float32)
    totals = np.zeros(2, np.uint32)
    rc = R.ref_pipeline(X, N, D, L, M, float(W), A, b, queries, Q, int(K), int(T), int(free_bytes),
                        buckets, ids, starts, sizes, codes, qb, kid, kd, totals)
    if rc != 0:
        raise RuntimeError(f"reference pipeline failed at stage {rc} (1 reset, 2 index, 3 search)")
    return {"index": Index(N, D, L, M, W, A, b, buckets, ids, starts, sizes, codes),
            "qbuckets": qb, "knn_ids": kid, "knn_dists": kd,
            "nonunique_total": int(totals[0]), "unique_total": int(totals[1])}


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            L.oracle_project.argtypes = [_f32p, _i64, _int, _f32p, _f32p, _int, _int, _flt, _f32p]
            L.oracle_bucket_table.argtypes = [_f32p, _i64, _int, _u32p, _u32p, _u32p, _f32p]
            L.oracle_bucket_table.restype = _i64
            L.oracle_index.argtypes = [_f32p, _int, _int, _int, _int, _flt, _f32p, _f32p,
                                       _u32p, _u32p, _u32p, _u32p, _f32p]
            L.oracle_probe_one.argtypes = [_f32p, _int, _int, _f32p]
            L.oracle_lookup_one.argtypes = [_f32p, _f32p, _i64, _int]
            L.oracle_lookup_one.restype = ctypes.c_int32
            L.oracle_search.argtypes = [_f32p, _int, _int, _int, _int, _flt, _f32p, _f32p,
                                        _u32p, _u32p, _u32p, _u32p, _f32p,
                                        _f32p, _int, _int, _int, _int,
                                        _i32p, _i32p, _f32p, _u64p, _u64p]
            L.oracle_topk.argtypes = [_u32p, _f32p, _i64, _int, _int, _i32p, _f32p]
            L.oracle_distance.argtypes = [_f32p, _f32p, _int]
            L.oracle_distance.restype = _flt
            L.oracle_exact_knn.argtypes = [_f32p, _int, _int, _f32p, _int, _int, _i32p, _f64p]
            L.oracle_save.argtypes = [ctypes.c_char_p, _int, _int, _int, _int, _flt, _f32p, _f32p,
                                      _u32p, _u32p, _u32p, _u32p, _f32p]
            L.oracle_save.restype = _int
            L.oracle_num_threads.restype = _int
            L.oracle_set_threads.argtypes = [_int]
            _lib = L
    return _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def num_threads() -> int:
    return lib().oracle_num_threads()


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def project(X, A, b, W):
    """Unfloored projections, shape [L*M, n]. X: [n, D]; A: [L, M, D]; b: [L, M]."""
    X = _c(X, np.float32)
    A = _c(A, np.float32)
    b = _c(b, np.float32)
    L, M, D = A.shape
    n = X.shape[0]
    out = np.empty((L * M, n), np.float32)
    lib().oracle_project(X, n, D, A, b, L, M, float(W), out)
    return out


class Index:
    """Oracle index: per-table totalIndices, startingIndices, sizes and codes."""

    def __init__(self, N, D, L, M, W, A, b, buckets, ids, starts, sizes, codes):
        self.N, self.D, self.L, self.M, self.W = N, D, L, M, float(W)
        self.A, self.b = A, b
        self.buckets = buckets      # [L] uint32
        self._ids, self._starts, self._sizes, self._codes = ids, starts, sizes, codes

    def ids(self, l):
        return self._ids[l]

    def starts(self, l):
        return self._starts[l, : self.buckets[l]]

    def sizes(self, l):
        return self._sizes[l, : self.buckets[l]]

    def codes(self, l):
        """[M, B] column-major bucket codes of table l (the reference layout)."""
        B = int(self.buckets[l])
        return self._codes[l, : B * self.M].reshape(self.M, B)

    def save(self, path):
        rc = lib().oracle_save(path.encode(), self.N, self.D, self.L, self.M, self.W,
                               _c(self.A, np.float32), _c(self.b, np.float32),
                               self.buckets, self._ids, self._starts, self._sizes, self._codes)
        if rc != 0:
            raise OSError(f"oracle_save failed for {path}")


def build_index(X, A, b, W) -> Index:
    """X: [N, D] float32; A: [L, M, D] (A[l] is the reference's D x M column-major);
    b: [L, M]."""
    X = _c(X, np.float32)
    A = _c(A, np.float32)
    b = _c(b, np.float32)
    L, M, D = A.shape
    N = X.shape[0]
    buckets = np.zeros(L, np.uint32)
    ids = np.zeros((L, N), np.uint32)
    starts = np.zeros((L, N), np.uint32)
    sizes = np.zeros((L, N), np.uint32)
    codes = np.zeros((L, N * M), np.float32)
    lib().oracle_index(X, N, D, L, M, float(W), A, b, buckets, ids, starts, sizes, codes)
    return Index(N, D, L, M, W, A, b, buckets, ids, starts, sizes, codes)


def probe_one(v, T):
    """Multiprobe code rows [T, M] of one query/table from its unfloored projection v[M]."""
    v = _c(v, np.float32)
    M = v.shape[0]
    rows = np.zeros((T, M), np.float32)
    lib().oracle_probe_one(v, M, int(T), rows)
    return rows


def search(index: Index, X, queries, K, T, tie_mode=0):
    """Returns dict with knn_ids [Q,K], knn_dists [Q,K], qbuckets [L, Q*T],
    nonunique [Q], unique [Q]."""
    X = _c(X, np.float32)
    queries = _c(queries, np.float32)
    Q = queries.shape[0]
    L = index.L
    qb = np.zeros((L, Q * T), np.int32)
    ids = np.zeros((Q, K), np.int32)
    d = np.zeros((Q, K), np.float32)
    nu = np.zeros(Q, np.uint64)
    un = np.zeros(Q, np.uint64)
    lib().oracle_search(X, index.N, index.D, L, index.M, index.W, _c(index.A, np.float32),
                        _c(index.b, np.float32), index.buckets, index._ids, index._starts,
                        index._sizes, index._codes, queries, Q, int(K), int(T), int(tie_mode),
                        qb, ids, d, nu, un)
    return {"knn_ids": ids, "knn_dists": d, "qbuckets": qb, "nonunique": nu, "unique": un}


def topk(cand, dist, K, tie_mode=0):
    """Top-K of unique candidates (ids ascending) -> (ids[K], dists[K])."""
    cand = _c(cand, np.uint32)
    dist = _c(dist, np.float32)
    ids = np.zeros(K, np.int32)
    d = np.zeros(K, np.float32)
    lib().oracle_topk(cand, dist, cand.shape[0], int(K), int(tie_mode), ids, d)
    return ids, d


def distance(q, x):
    q = _c(q, np.float32)
    x = _c(x, np.float32)
    return float(lib().oracle_distance(q, x, q.shape[0]))


def exact_knn(X, queries, K):
    X = _c(X, np.float32)
    queries = _c(queries, np.float32)
    Q, D = queries.shape
    ids = np.zeros((Q, K), np.int32)
    d = np.zeros((Q, K), np.float64)
    lib().oracle_exact_knn(X, X.shape[0], D, queries, Q, int(K), ids, d)
    return ids, d
