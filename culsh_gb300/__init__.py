"""culsh_gb300: GB300-native Euclidean LSH index build and k-NN search.

Python mirror of the reference's ``cuLSH::HashTables`` / ``cuLSH::SearchTables``
API (cuLSH_HashTables.cu, cuLSH_SearchTables.cu) over the C ABI of
``libculsh.so`` (``include/culsh.h``). Same method names and argument meaning;
failures raise :class:`CulshError` carrying the library's status code and
message instead of returning ``False``.

Arrays follow the reference's layouts expressed as C-contiguous numpy arrays:
the dataset / queries (D x N column-major) are ``[N, D]``, ``A[l]`` (D x M
column-major) is ``[M, D]``, bucket codes (B x M column-major) are ``[M, B]``,
kNN ids / distances (K x Q) are ``[Q, K]``, query buckets (Q x T) ``[Q, T]``.

There is no CPU fallback: every compute call goes through the CUDA library,
and importing fails loudly when the library has not been built.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libculsh.so")

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_STATE = 2
ERR_CUDA = 3
ERR_OUT_OF_MEMORY = 4
ERR_IO = 5
ERR_NUMERIC = 6
ERR_CAPACITY = 7
ERR_DEVICE = 8
ERR_FORMAT = 9
PENDING = 10

MAX_M = 64
MAX_T = 256
MAX_K = 2048


class CulshError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[culsh error {code}] {message}")
        self.code = code


class _Times(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("buckets", "collect", "sort", "unique", "distances", "knn")]


class _Profile(ctypes.Structure):
    _fields_ = [("project_ms", ctypes.c_float), ("probe_ms", ctypes.c_float), ("candidates_ms", ctypes.c_float),
                ("launches", ctypes.c_int), ("deferred_queries", ctypes.c_int), ("key_words", ctypes.c_int),
                ("candidates_mode", ctypes.c_int), ("graph_mode", ctypes.c_int), ("rechecked", ctypes.c_longlong),
                ("dense_queries", ctypes.c_int), ("host_path", ctypes.c_int), ("stage_times", ctypes.c_int),
                ("knn_queries", ctypes.c_int), ("knn_fallback", ctypes.c_int),
                ("membership_ms", ctypes.c_float), ("knn_ms", ctypes.c_float), ("bucket_rows", ctypes.c_int)]


class _Tuning(ctypes.Structure):
    _fields_ = [("proj_tile", ctypes.c_int), ("probe_batch", ctypes.c_int), ("candidates_mode", ctypes.c_int),
                ("ws_threads", ctypes.c_int), ("ws_blocks_per_sm", ctypes.c_int), ("ws_chunk", ctypes.c_int),
                ("distance_bf16", ctypes.c_int), ("ws_set_slots", ctypes.c_int), ("search_ms", ctypes.c_float),
                ("configs_tried", ctypes.c_int), ("probe_split", ctypes.c_int), ("ws_order", ctypes.c_int),
                ("dense_tc", ctypes.c_int), ("dense_min", ctypes.c_int)]


class _IndexProfile(ctypes.Structure):
    _fields_ = [("project_ms", ctypes.c_float), ("pack_ms", ctypes.c_float), ("sort_ms", ctypes.c_float),
                ("bucket_ms", ctypes.c_float), ("total_ms", ctypes.c_float), ("tensor_cores", ctypes.c_int),
                ("recomputed", ctypes.c_longlong), ("key_words", ctypes.c_int), ("sort_passes", ctypes.c_int),
                ("sort_form", ctypes.c_int)]


class _ServerConfig(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_int), ("max_batch_queries", ctypes.c_int), ("memory_budget", ctypes.c_longlong),
                ("graphs", ctypes.c_int)]


class _ServerStats(ctypes.Structure):
    _fields_ = [("requests", ctypes.c_longlong), ("queries", ctypes.c_longlong), ("batches", ctypes.c_longlong),
                ("failed", ctypes.c_longlong), ("wall_s", ctypes.c_double), ("qps", ctypes.c_double),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double), ("max_in_flight", ctypes.c_int), ("slots", ctypes.c_int),
                ("peak_device_bytes", ctypes.c_longlong), ("budget_bytes", ctypes.c_longlong)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_FP = ctypes.POINTER(ctypes.c_float)
_UP = ctypes.POINTER(ctypes.c_uint)
_IP = ctypes.POINTER(ctypes.c_int)

# name -> (restype, argtypes); the complete exported surface of include/culsh.h
ABI = {
    "culsh_last_error": (ctypes.c_char_p, []),
    "culsh_version": (_I, []),
    "culsh_index_create": (_I, [ctypes.POINTER(_P)]),
    "culsh_index_destroy": (None, [_P]),
    "culsh_index_reset_random": (_I, [_P, _I, _I, _I, _I, _F, ctypes.c_ulonglong, _P]),
    "culsh_index_reset": (_I, [_P, _I, _I, _I, _I, _F, ctypes.POINTER(_FP), ctypes.POINTER(_FP), _P]),
    "culsh_index_build": (_I, [_P, _P, _P]),
    "culsh_index_build_device": (_I, [_P, _P, _P]),
    "culsh_index_save": (_I, [_P, ctypes.c_char_p, _P]),
    "culsh_index_load": (_I, [_P, ctypes.c_char_p, _P]),
    "culsh_index_params": (None, [_P, _IP, _IP, _IP, _IP, _FP]),
    "culsh_index_A": (_FP, [_P, _I]),
    "culsh_index_b": (_FP, [_P, _I]),
    "culsh_index_bucket_count": (ctypes.c_uint, [_P, _I]),
    "culsh_index_bucket_counts": (_UP, [_P]),
    "culsh_index_total_indices": (_UP, [_P, _I]),
    "culsh_index_starting_indices": (_UP, [_P, _I]),
    "culsh_index_sizes": (_UP, [_P, _I]),
    "culsh_index_codes": (_FP, [_P, _I]),
    "culsh_index_profile_get": (_I, [_P, ctypes.POINTER(_IndexProfile)]),
    "culsh_search_create": (_I, [ctypes.POINTER(_P)]),
    "culsh_search_destroy": (None, [_P]),
    "culsh_search_reset": (_I, [_P, _P, _I, _I]),
    "culsh_search_run": (_I, [_P, _P, _I, _P, _P]),
    "culsh_search_run_device": (_I, [_P, _P, _I, _P, _P, _P]),
    "culsh_search_knn_ids": (_IP, [_P]),
    "culsh_search_knn_distances": (_FP, [_P]),
    "culsh_search_query_buckets": (_IP, [_P, _I]),
    "culsh_search_selectivity": (_F, [_P]),
    "culsh_search_nonunique_percentage": (_F, [_P]),
    "culsh_search_total_unique": (ctypes.c_ulonglong, [_P]),
    "culsh_search_total_nonunique": (ctypes.c_ulonglong, [_P]),
    "culsh_search_times": (None, [_P, ctypes.POINTER(_Times)]),
    "culsh_search_profile_get": (_I, [_P, ctypes.POINTER(_Profile)]),
    "culsh_search_run_device_noalloc": (_I, [_P, _P, _I, _P, _P, _P]),
    "culsh_search_autotune": (_I, [_P, _P, _I, _P, _P, _P, ctypes.POINTER(_Tuning)]),
    "culsh_search_get_tuning": (_I, [_P, ctypes.POINTER(_Tuning)]),
    "culsh_search_set_tuning": (_I, [_P, ctypes.POINTER(_Tuning)]),
    "culsh_search_set_graphs": (_I, [_P, _I]),
    "culsh_search_set_profiling": (_I, [_P, _I]),
    "culsh_search_device_bytes": (ctypes.c_longlong, [_P]),
    "culsh_search_estimate_bytes": (ctypes.c_longlong, [_P, _I, _I, _I]),
    "culsh_search_release": (_I, [_P]),
    "culsh_server_create": (_I, [ctypes.POINTER(_P), _P, ctypes.POINTER(_ServerConfig)]),
    "culsh_server_submit": (_I, [_P, _P, _I, _I, _I, _P, _P, ctypes.POINTER(ctypes.c_ulonglong)]),
    "culsh_server_wait": (_I, [_P, ctypes.c_ulonglong, ctypes.c_double]),
    "culsh_server_stats_get": (_I, [_P, ctypes.POINTER(_ServerStats)]),
    "culsh_server_stats_reset": (_I, [_P]),
    "culsh_server_destroy": (None, [_P]),
}

_lib = None


def lib():
    """The loaded libculsh (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in ABI.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int):
    if rc != OK:
        raise CulshError(rc, lib().culsh_last_error().decode(errors="replace"))


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def _copy_out(ptr, n, dtype):
    if not ptr or n == 0:
        return None if not ptr else np.zeros(0, dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class HashTables:
    """cuLSH::HashTables (cuLSH_HashTables.cu:51-108)."""

    def __init__(self):
        self._h = ctypes.c_void_p()
        _check(lib().culsh_index_create(ctypes.byref(self._h)))
        self._X_keep = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.culsh_index_destroy(h)
            self._h = None

    # cuLSH_HashTables.cu:190-249
    def reset(self, N_or_filename, D=None, L=None, M=None, W=None, A=None, b=None, seed=None):
        if isinstance(N_or_filename, (str, bytes, os.PathLike)):
            return self.load(N_or_filename)
        N = int(N_or_filename)
        if A is None:
            s = int(seed) if seed is not None else int.from_bytes(os.urandom(8), "little")
            _check(lib().culsh_index_reset_random(self._h, N, int(D), int(L), int(M), float(W), s, None))
            return
        A = _f32(A)
        b = _f32(b)
        L, M, D = int(L), int(M), int(D)
        if A.shape != (L, M, D) or b.shape != (L, M):
            raise CulshError(ERR_INVALID_ARGUMENT, f"A must be [L, M, D] = {(L, M, D)}, b [L, M]; got {A.shape}, {b.shape}")
        Ap = (_FP * L)(*[A[l].ctypes.data_as(_FP) for l in range(L)])
        bp = (_FP * L)(*[b[l].ctypes.data_as(_FP) for l in range(L)])
        _check(lib().culsh_index_reset(self._h, N, D, L, M, float(W), Ap, bp, None))

    # cuLSH_HashTables.cu:486-520
    def index(self, matrix):
        X = _f32(matrix)
        N, D = self.getN(), self.getD()
        if X.size != N * D:
            raise CulshError(ERR_INVALID_ARGUMENT, f"dataset has {X.size} floats, expected N*D = {N * D}")
        self._X_keep = X   # the device copy is keyed by this host pointer
        _check(lib().culsh_index_build(self._h, _ptr(X), None))

    def index_device(self, d_ptr: int, stream: int = 0):
        """Build from a device-resident dataset (borrowed, not copied)."""
        _check(lib().culsh_index_build_device(self._h, ctypes.c_void_p(d_ptr), ctypes.c_void_p(stream or None)))

    def save(self, filename):
        _check(lib().culsh_index_save(self._h, os.fsencode(filename), None))

    def load(self, filename):
        _check(lib().culsh_index_load(self._h, os.fsencode(filename), None))

    def _params(self):
        v = [ctypes.c_int() for _ in range(4)]
        w = ctypes.c_float()
        lib().culsh_index_params(self._h, *[ctypes.byref(x) for x in v], ctypes.byref(w))
        return [x.value for x in v] + [w.value]

    def getN(self): return self._params()[0]
    def getD(self): return self._params()[1]
    def getL(self): return self._params()[2]
    def getM(self): return self._params()[3]
    def getW(self): return self._params()[4]

    def getA(self, table):
        N, D, L, M, W = self._params()
        a = _copy_out(lib().culsh_index_A(self._h, table), D * M, np.float32)
        return None if a is None else a.reshape(M, D)

    def getb(self, table):
        return _copy_out(lib().culsh_index_b(self._h, table), self.getM(), np.float32)

    def getBuckets(self, table=None):
        if table is None:
            return _copy_out(lib().culsh_index_bucket_counts(self._h), self.getL(), np.uint32)
        return int(lib().culsh_index_bucket_count(self._h, table))

    def getBuckets_totalIndices(self, table):
        return _copy_out(lib().culsh_index_total_indices(self._h, table), self.getN(), np.uint32)

    def getBuckets_startingIndices(self, table):
        return _copy_out(lib().culsh_index_starting_indices(self._h, table), self.getBuckets(table), np.uint32)

    def getBuckets_sizes(self, table):
        return _copy_out(lib().culsh_index_sizes(self._h, table), self.getBuckets(table), np.uint32)

    def profile(self):
        """Per-stage device milliseconds of the last device index build."""
        p = _IndexProfile()
        _check(lib().culsh_index_profile_get(self._h, ctypes.byref(p)))
        return {n: getattr(p, n) for n, _ in _IndexProfile._fields_}

    def getBuckets_codes(self, table):
        B, M = self.getBuckets(table), self.getM()
        c = _copy_out(lib().culsh_index_codes(self._h, table), B * M, np.float32)
        return None if c is None else c.reshape(M, B)


class SearchTables:
    """cuLSH::SearchTables (cuLSH_SearchTables.cu:42-107)."""

    def __init__(self):
        self._h = ctypes.c_void_p()
        _check(lib().culsh_search_create(ctypes.byref(self._h)))
        self._ht = None
        self.K = self.T = self.Q = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.culsh_search_destroy(h)
            self._h = None

    def reset(self, hashtables: HashTables, K: int, T: int = 1):
        self._ht = hashtables
        self.K, self.T = int(K), int(T)
        _check(lib().culsh_search_reset(self._h, hashtables._h if hashtables else None, self.K, self.T))

    def search(self, queries, Q=None, dataset=None):
        q = _f32(queries)
        D = self._ht.getD()
        Q = int(Q if Q is not None else q.size // D)
        if q.size < Q * D:
            raise CulshError(ERR_INVALID_ARGUMENT, "queries array is smaller than Q*D")
        ds = None
        if dataset is not None:
            ds = _f32(dataset)
            if ds is not self._ht._X_keep and self._ht._X_keep is not None and ds.ctypes.data != self._ht._X_keep.ctypes.data:
                self._ds_keep = ds
        _check(lib().culsh_search_run(self._h, _ptr(q), Q, _ptr(ds) if ds is not None else None, None))
        self.Q = Q

    def search_device(self, d_queries: int, Q: int, d_ids: int, d_dists: int, stream: int = 0):
        _check(lib().culsh_search_run_device(self._h, ctypes.c_void_p(d_queries), int(Q), ctypes.c_void_p(d_ids),
                                             ctypes.c_void_p(d_dists), ctypes.c_void_p(stream or None)))
        self.Q = int(Q)

    def autotune(self, d_queries: int, Q: int, d_ids: int, d_dists: int, stream: int = 0):
        """Times the search over its tuning space on these device queries and
        keeps the fastest configuration; returns it as a dict."""
        t = _Tuning()
        _check(lib().culsh_search_autotune(self._h, ctypes.c_void_p(d_queries), int(Q), ctypes.c_void_p(d_ids),
                                           ctypes.c_void_p(d_dists), ctypes.c_void_p(stream or None), ctypes.byref(t)))
        self.Q = int(Q)
        return {n: getattr(t, n) for n, _ in _Tuning._fields_}

    def get_tuning(self):
        t = _Tuning()
        _check(lib().culsh_search_get_tuning(self._h, ctypes.byref(t)))
        return {n: getattr(t, n) for n, _ in _Tuning._fields_}

    def set_tuning(self, **kw):
        """Sets tuning fields (proj_tile, probe_batch, probe_split,
        candidates_mode, ws_threads, ws_blocks_per_sm, ws_chunk,
        distance_bf16, ws_set_slots, ws_order, dense_tc, dense_min); others keep
        their value."""
        t = _Tuning()
        _check(lib().culsh_search_get_tuning(self._h, ctypes.byref(t)))
        for k, v in kw.items():
            if k not in dict(_Tuning._fields_):
                raise KeyError(k)
            setattr(t, k, v)
        _check(lib().culsh_search_set_tuning(self._h, ctypes.byref(t)))

    def set_graphs(self, enabled: bool):
        _check(lib().culsh_search_set_graphs(self._h, 1 if enabled else 0))

    def set_profiling(self, stage_times: bool):
        """Stage timing events on (default) or off (a few microseconds less
        device time per search; stage times then read 0)."""
        _check(lib().culsh_search_set_profiling(self._h, 1 if stage_times else 0))

    def getKnnIds(self):
        a = _copy_out(lib().culsh_search_knn_ids(self._h), self.Q * self.K, np.int32)
        return None if a is None else a.reshape(self.Q, self.K)

    def getKnnDistances(self):
        a = _copy_out(lib().culsh_search_knn_distances(self._h), self.Q * self.K, np.float32)
        return None if a is None else a.reshape(self.Q, self.K)

    def getQueryBuckets(self, table):
        a = _copy_out(lib().culsh_search_query_buckets(self._h, table), self.Q * self.T, np.int32)
        return None if a is None else a.reshape(self.Q, self.T)

    def getSelectivity(self):
        return float(lib().culsh_search_selectivity(self._h))

    def getNonUniquePercentage(self):
        return float(lib().culsh_search_nonunique_percentage(self._h))

    def getTotalCandidates_unique(self):
        return int(lib().culsh_search_total_unique(self._h))

    def getTotalCandidates_nonUnique(self):
        return int(lib().culsh_search_total_nonunique(self._h))

    def getTimes(self):
        t = _Times()
        lib().culsh_search_times(self._h, ctypes.byref(t))
        return {n: getattr(t, n) for n, _ in _Times._fields_}

    def profile(self):
        """Per-stage device milliseconds and launch count of the last search."""
        p = _Profile()
        _check(lib().culsh_search_profile_get(self._h, ctypes.byref(p)))
        return {n: getattr(p, n) for n, _ in _Profile._fields_}


class Server:
    """Serving loop over one device-resident index (culsh_server_*): requests
    of any Q, K, T are batched as slots and device memory free up, and run
    concurrently on the device; each returns what a lone search returns."""

    def __init__(self, hashtables: HashTables, slots: int = 4, max_batch_queries: int = 8192,
                 memory_budget: int = 0, graphs: bool = False):
        self._ht = hashtables
        self._h = ctypes.c_void_p()
        cfg = _ServerConfig(int(slots), int(max_batch_queries), int(memory_budget), 1 if graphs else 0)
        _check(lib().culsh_server_create(ctypes.byref(self._h), hashtables._h, ctypes.byref(cfg)))
        self._keep = {}

    def submit(self, queries, K: int, T: int = 1) -> int:
        """Queues queries [Q, D]; returns a ticket for wait()."""
        q = _f32(queries).reshape(-1, self._ht.getD())
        Q = q.shape[0]
        ids = np.empty((Q, int(K)), np.int32)
        d = np.empty((Q, int(K)), np.float32)
        t = ctypes.c_ulonglong()
        _check(lib().culsh_server_submit(self._h, _ptr(q), Q, int(K), int(T), ids.ctypes.data_as(_P),
                                         d.ctypes.data_as(_P), ctypes.byref(t)))
        self._keep[t.value] = (q, ids, d)
        return t.value

    def wait(self, ticket: int, timeout: float = -1.0):
        """(ids [Q, K], dists [Q, K]) of a request; raises CulshError on its error."""
        rc = lib().culsh_server_wait(self._h, ctypes.c_ulonglong(ticket), float(timeout))
        if rc == PENDING:
            raise TimeoutError(f"request {ticket} still running")
        _, ids, d = self._keep.pop(ticket)
        _check(rc)
        return ids, d

    def stats(self):
        st = _ServerStats()
        _check(lib().culsh_server_stats_get(self._h, ctypes.byref(st)))
        return {n: getattr(st, n) for n, _ in _ServerStats._fields_}

    def reset_stats(self):
        _check(lib().culsh_server_stats_reset(self._h))

    def close(self):
        if self._h and self._h.value and _lib is not None:
            _lib.culsh_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
