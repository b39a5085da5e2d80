/*
 * culsh.h - C ABI of libculsh, a GB300-native (sm_103a) Euclidean LSH index
 * and k-nearest-neighbour search with the behaviour of cuLSH (ariskag/cuLSH).
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes. Every
 * entry point replaces one member of the reference's header-only C++ classes
 * cuLSH::HashTables (cuLSH_HashTables.cu) and cuLSH::SearchTables
 * (cuLSH_SearchTables.cu); the citation beside each one names the member.
 * The drop-in C++ classes in cuLSH.h are thin inline wrappers over this ABI.
 *
 * Conventions (identical to the reference):
 *   dataset X  : D x N float, column-major (point n is X[n*D .. n*D+D))
 *   queries    : D x Q float, column-major
 *   A[l]       : D x M float, column-major (column m is A[l][m*D .. m*D+D)); b[l]: M floats
 *   knn ids    : K x Q int, column-major (query q is ids[q*K .. q*K+K)), -1 = no neighbour
 *   knn dists  : K x Q float, SQUARED Euclidean distances, FLT_MAX = no neighbour
 *   query buckets of table l: Q x T int, entry q*T+t (probe t of query q), -1 = no bucket
 *
 * Status codes: 0 on success, a CULSH_ERR_* value otherwise; culsh_last_error()
 * returns the message of the last failure on the calling thread.
 * Objects are not thread-safe; calls on one object are synchronous.
 */
#ifndef CULSH_C_ABI_H
#define CULSH_C_ABI_H

#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CULSH_OK 0
#define CULSH_ERR_INVALID_ARGUMENT 1 /* a parameter is out of its domain               */
#define CULSH_ERR_STATE 2            /* call order violated (e.g. search before index)  */
#define CULSH_ERR_CUDA 3             /* a CUDA runtime call failed                       */
#define CULSH_ERR_OUT_OF_MEMORY 4    /* host or device allocation failed / admission    */
#define CULSH_ERR_IO 5               /* file could not be opened, read or written        */
#define CULSH_ERR_NUMERIC 6          /* non-finite projection or code beyond int32       */
#define CULSH_ERR_CAPACITY 7         /* size beyond a documented limit of this library   */
#define CULSH_ERR_DEVICE 8           /* a device-side bounded wait or insert gave up     */
#define CULSH_ERR_FORMAT 9           /* index file truncated or inconsistent             */
#define CULSH_PENDING 10             /* serving: the request has not completed (no error) */

/* Limits of this implementation (the reference has the memory limits only). */
#define CULSH_MAX_M 64      /* projection columns per table               */
#define CULSH_MAX_T 256     /* probes per table and query                 */
#define CULSH_MAX_K 2048    /* neighbours per query                       */
#define CULSH_MAX_N ((1 << 30) - 1)

typedef struct culsh_index culsh_index;   /* cuLSH::HashTables  (cuLSH_HashTables.cu:51-108)  */
typedef struct culsh_search culsh_search; /* cuLSH::SearchTables (cuLSH_SearchTables.cu:42-107) */

/* cuLSH::SearchTables::timesStruct (cuLSH_SearchTables.cu:44-52), seconds. */
typedef struct culsh_times {
    float buckets;   /* query projection, multiprobe codes and bucket lookup           */
    float collect;   /* fused into `distances` (0)                                       */
    float sort;      /* fused into `distances` (0)                                       */
    float unique;    /* fused into `distances` (0)                                       */
    float distances; /* candidate gather, dedup, distances and top-K (one fused kernel)  */
    float knn;       /* copy of the K x Q results back to the host                       */
} culsh_times;

const char* culsh_last_error(void);
int culsh_version(void);

/* ---- HashTables ---------------------------------------------------------- */
int culsh_index_create(culsh_index** out);          /* HashTables::HashTables  cuLSH_HashTables.cu:111-119 */
void culsh_index_destroy(culsh_index* ix);          /* HashTables::~HashTables cuLSH_HashTables.cu:78 */

/* HashTables::reset(N,D,L,M,W,dbg) cuLSH_HashTables.cu:190-210: random A ~ N(0,1),
 * b = W*(u - min u), u ~ U(0,1] per table, from a seeded counter-based generator
 * (the reference seeds cuRAND with time(0)). */
int culsh_index_reset_random(culsh_index* ix, int N, int D, int L, int M, float W, unsigned long long seed,
                             FILE* dbg);
/* HashTables::reset(N,D,L,M,W,A,b,dbg) cuLSH_HashTables.cu:213-241: A and b are copied. */
int culsh_index_reset(culsh_index* ix, int N, int D, int L, int M, float W, const float* const* A,
                      const float* const* b, FILE* dbg);
/* HashTables::index(matrix,dbg) cuLSH_HashTables.cu:486-520. X (host, D x N) is
 * copied to the device and kept there for later searches. */
int culsh_index_build(culsh_index* ix, const float* X, FILE* dbg);
/* Device-resident variant of index(): d_X is a device pointer that stays
 * borrowed (not copied) until the next build, reset or destroy. stream: a
 * cudaStream_t, NULL = the object's own stream. */
int culsh_index_build_device(culsh_index* ix, const float* d_X, void* stream);
/* HashTables::save / load cuLSH_HashTables.cu:395-483 (identical file layout);
 * HashTables::reset(filename,dbg) cuLSH_HashTables.cu:243-249 is load(). */
int culsh_index_save(culsh_index* ix, const char* path, FILE* dbg);
int culsh_index_load(culsh_index* ix, const char* path, FILE* dbg);

/* Getters cuLSH_HashTables.cu:89-103. Pointers stay valid until the next
 * reset/index/load/destroy; NULL (or 0) when unset. */
void culsh_index_params(const culsh_index* ix, int* N, int* D, int* L, int* M, float* W);
const float* culsh_index_A(culsh_index* ix, int table);
const float* culsh_index_b(culsh_index* ix, int table);
unsigned culsh_index_bucket_count(culsh_index* ix, int table);
const unsigned* culsh_index_bucket_counts(culsh_index* ix);
const unsigned* culsh_index_total_indices(culsh_index* ix, int table);
const unsigned* culsh_index_starting_indices(culsh_index* ix, int table);
const unsigned* culsh_index_sizes(culsh_index* ix, int table);
const float* culsh_index_codes(culsh_index* ix, int table);

/* Measurement aid with no counterpart in the reference: device time of each
 * stage of the last device index build (CUDA events on its stream). */
typedef struct culsh_index_profile {
    float project_ms;      /* projection + codes (tensor-core or FP32 SIMT kernel) */
    float pack_ms;         /* packing codes into sort keys                         */
    float sort_ms;         /* radix sort of all tables                             */
    float bucket_ms;       /* run-length bucketing + hash build                    */
    float total_ms;
    int tensor_cores;      /* 1 when the tcgen05 projection produced the codes     */
    long long recomputed;  /* codes its error bound left to the FP32 recomputation */
    int key_words;         /* 32-bit words of a packed bucket key                  */
    int sort_passes;       /* 8-bit digit passes over the keys                     */
    int sort_form;         /* 1: passes over the top key word, then each run of    */
                           /* equal top words ordered by its lower words and id;   */
                           /* 2: that form met a run too long and sorted all words */
                           /* again; 0: passes over all words (one-word keys)      */
} culsh_index_profile;
int culsh_index_profile_get(culsh_index* ix, culsh_index_profile* out);

/* ---- SearchTables -------------------------------------------------------- */
int culsh_search_create(culsh_search** out);        /* SearchTables::SearchTables  cuLSH_SearchTables.cu:112-122 */
void culsh_search_destroy(culsh_search* s);         /* SearchTables::~SearchTables cuLSH_SearchTables.cu:74 */
/* SearchTables::reset(hashtables,K,T) cuLSH_SearchTables.cu:127-139 (ix is not owned). */
int culsh_search_reset(culsh_search* s, culsh_index* ix, int K, int T);
/* SearchTables::search(queries,Q,dataset,dbg) cuLSH_SearchTables.cu:197-463.
 * dataset must be the indexed dataset; when it is the pointer given to
 * culsh_index_build (or NULL after a build) the device copy is reused. */
int culsh_search_run(culsh_search* s, const float* queries, int Q, const float* dataset, FILE* dbg);
/* Device-resident variant: d_queries (D x Q) in device memory, results written
 * to the caller's device buffers d_ids / d_dists (K x Q). */
int culsh_search_run_device(culsh_search* s, const float* d_queries, int Q, int* d_ids, float* d_dists,
                            void* stream);

/* Search-path tuning (no counterpart in the reference). The search runs as a
 * CUDA graph captured on first use and replayed while the query pointer,
 * count, outputs, index buffers and tuning stay the same (captured again
 * otherwise); graphs are used on any stream but the legacy default stream
 * and never inside a caller's own capture. */
typedef struct culsh_tuning {
    int proj_tile;        /* query projection tiling (points x columns per block): 0 (64x128),
                             1 (32x128), 2 (128x64), 3 (64x64), 4 (32x64)               */
    int probe_batch;      /* multiprobe hash-group loads in flight per thread: 1, 2, 4   */
    int candidates_mode;  /* 0: one block per query; 1: persistent work-stealing grid   */
    int ws_threads;       /* work-stealing threads per item: 64, 128, 256, 512          */
    int ws_blocks_per_sm; /* resident work-stealing CTAs per SM, 0 = occupancy limit     */
    int ws_chunk;         /* non-unique candidates per id partition (64 .. 65536)        */
    int distance_bf16;    /* 1: candidate distances from a bf16 copy of the dataset, then
                             an exact FP32 rerank of every candidate the proven error
                             bound cannot exclude (same results as 0)                  */
    int ws_set_slots;     /* work-stealing shared hash set per item: 4096, 8192 or 16384 slots */
    float search_ms;      /* culsh_search_autotune: median device ms of the choice       */
    int configs_tried;    /* culsh_search_autotune: configurations timed                 */
    int probe_split;      /* M <= 16: 1 enumerate every probe first, then look each up in
                             its own thread behind a key filter; 2 look a pair's probes
                             up behind the filter at the end of its enumeration
                             (same results as 0)                                        */
    int ws_order;         /* 1: work-stealing items planned in the locality order of the
                             queries' home buckets, so queries that share candidates run
                             together and share rows in L2 (same results as 0)         */
    int dense_tc;         /* 1: dense queries (see dense_min) take the tensor-core path:
                             an N-bit candidate membership row per query, then q.x for
                             all points by tcgen05 GEMM tiles with the top-K kept in the
                             epilogue, exact distances (same results as 0); 0: the SIMT
                             bitmap kernel                                              */
    int dense_min;        /* non-unique candidates from which a query is dense; 0: the
                             default, max(4096, N/256) for the tensor-core path and
                             max(32768, N/16) for the SIMT bitmap kernel               */
} culsh_tuning;

/* Times the search over the tuning space on the caller's queries (device
 * buffers, as culsh_search_run_device) and keeps the fastest configuration
 * for later searches of this object. Every configuration must return the
 * same ids, distances and counts, else CULSH_ERR_DEVICE. */
int culsh_search_autotune(culsh_search* s, const float* d_queries, int Q, int* d_ids, float* d_dists,
                          void* stream, culsh_tuning* out);
int culsh_search_get_tuning(culsh_search* s, culsh_tuning* out);
int culsh_search_set_tuning(culsh_search* s, const culsh_tuning* in);   /* CULSH_ERR_INVALID_ARGUMENT when out of range */
int culsh_search_set_graphs(culsh_search* s, int enabled);               /* default 1 */
/* Stage timing (default 1): four events in each search (the per-stage times
 * of culsh_search_profile_get and culsh_search_get_times). Each costs a few
 * microseconds of device time in the graph; 0 leaves them out, and the stage
 * times then read 0 (profile.stage_times = 0). The autotuner turns them on
 * while it runs. */
int culsh_search_set_profiling(culsh_search* s, int stage_times);

/* Device memory of a search object (no counterpart in the reference; the
 * serving loop's admission uses them). device_bytes: bytes its buffers hold
 * now (they grow to the largest search and are kept for reuse);
 * estimate_bytes: an upper bound on what one device search of Q queries with
 * K, T makes them hold; release: frees them (and the cached graph). */
long long culsh_search_device_bytes(culsh_search* s);
long long culsh_search_estimate_bytes(const culsh_index* ix, int Q, int K, int T);
int culsh_search_release(culsh_search* s);

/* Getters cuLSH_SearchTables.cu:83-105. */
const int* culsh_search_knn_ids(culsh_search* s);
const float* culsh_search_knn_distances(culsh_search* s);
const int* culsh_search_query_buckets(culsh_search* s, int table);
float culsh_search_selectivity(culsh_search* s);
float culsh_search_nonunique_percentage(culsh_search* s);
unsigned long long culsh_search_total_unique(culsh_search* s);
unsigned long long culsh_search_total_nonunique(culsh_search* s);
void culsh_search_times(culsh_search* s, culsh_times* out);

/* Measurement aid with no counterpart in the reference: device time of each
 * stage of the last search (CUDA events on the launching stream) and the
 * number of kernels it launched. */
typedef struct culsh_search_profile {
    float project_ms;    /* query projection onto all L*M columns             */
    float probe_ms;      /* multiprobe codes + hash lookup + non-unique counts */
    float candidates_ms; /* gather + dedup + distances + top-K (incl. re-runs) */
    int launches;        /* kernels launched by libculsh in the last search    */
    int deferred_queries;/* queries re-run after growing the overflow arena    */
    int key_words;       /* 32-bit words of a packed bucket key (index layout) */
    int candidates_mode; /* 0: one block per query; 1: persistent work-stealing
                            grid over id partitions; 2: work-stealing, re-run
                            per query after a partition overflowed            */
    int graph_mode;      /* 0: direct launches; 1: graph captured; 2: replayed */
    long long rechecked; /* BF16 distance form: candidates re-read in FP32     */
    int dense_queries;   /* queries deduplicated in an N-bit bitmap (candidate
                            sets of at least max(32768, N/16) ids)             */
    int host_path;       /* 0: device buffers (culsh_search_run_device*);
                            1: host buffers staged through device copies;
                            2: host buffers read and written by the kernels
                            directly (device with pageable memory access,
                            16-byte aligned queries), a copy kernel moving
                            the queries to the device; 3: as 2, with the
                            projection reading the queries and writing them
                            to the device on the way (L*M <= 192)            */
    int stage_times;     /* 1: the stage times above were measured; 0: stage
                            events off (culsh_search_set_profiling)          */
    int knn_queries;     /* dense queries served by the tensor-core path     */
    int knn_fallback;    /* of those, queries whose bound-form lists could not
                            prove the top-K, re-run by the exact per-query
                            kernel                                          */
    float membership_ms; /* tensor-core path, stage times: planning and the
                            candidate membership rows ...                   */
    float knn_ms;        /* ... and the tensor-core distances, top-K lists
                            and merge (0 unless measured)                   */
    int bucket_rows;     /* tensor-core path: index buckets kept as N-bit rows
                            and ORed whole into the membership rows (buckets
                            of at least max(1024, N/64) ids); 0: none       */
} culsh_search_profile;
int culsh_search_profile_get(culsh_search* s, culsh_search_profile* out);

/* Same search as culsh_search_run_device, for callers that cannot allocate
 * device memory (a locked-down or externally owned allocator, no allocation
 * allowed on a latency-critical path). No counterpart in the reference. It
 * calls no cudaMalloc/cudaFree and creates no stream or event: its scratch is
 * a fixed 64 MiB __device__ array inside libculsh, reserved on every GPU that
 * loads the library until the process exits. Requirements and limits:
 *  - the index is already resident on the device (after index(), or after one
 *    ordinary search of a loaded index), else CULSH_ERR_STATE;
 *  - Q*(4*L*M + 4*L*T + 24) bytes plus a 1 MiB overflow arena must fit in the
 *    64 MiB (Q = 10,000 with L=16, M=12, T=16 uses 18 MB), else
 *    CULSH_ERR_CAPACITY; a single query's candidate set must fit the arena;
 *  - the first call on a device looks up the array's address: make it before
 *    any stream capture; the address is kept for the process, so a
 *    cudaDeviceReset while the library is loaded is not supported;
 *  - the call synchronises `stream` and returns when d_ids / d_dists hold the
 *    results (it reads counters back to admit large candidate sets in rounds);
 *  - calls share the array: calls that overlap on the GPU race, serialise them;
 *  - stream NULL is the legacy default stream; the search object's getters
 *    are not updated (results go only to d_ids / d_dists). */
int culsh_search_run_device_noalloc(culsh_search* s, const float* d_queries, int Q, int* d_ids, float* d_dists,
                                    void* stream);

/* ---------------------------------------------------------------------------
 * Serving loop (no counterpart in the reference, whose search is one blocking
 * call per query set, cuLSH_SearchTables.cu:197-463). A server keeps one index
 * resident and runs kNN requests of any Q, K, T as they arrive: a scheduler
 * merges pending requests with the same (K, T) into batches (continuous
 * batching) and hands each batch to a free slot (a search object with its own
 * stream and worker thread), so batches overlap on the device. A batch is
 * admitted when the device bytes of all slots stay within the memory budget;
 * a request that alone exceeds it fails with CULSH_ERR_OUT_OF_MEMORY. Every
 * request gets exactly the ids and distances it gets when searched alone.
 * The index must not be rebuilt, reset or destroyed while a server uses it;
 * its dataset must be on the device (after index(), or after one search with
 * the dataset following a load()). */
typedef struct culsh_server culsh_server;
typedef struct culsh_server_config {
    int slots;                /* batches on the device at once, 1..64 (0: 4)          */
    int max_batch_queries;    /* queries merged into one batch (0: 8192)              */
    long long memory_budget;  /* device bytes for all slots (0: 80% of free memory)   */
    int graphs;               /* 1: slots replay CUDA graphs of their searches (pays off
                                 when batch sizes repeat); 0: direct launches, since a
                                 new batch size would re-capture the graph             */
} culsh_server_config;
typedef struct culsh_server_stats {
    long long requests;       /* completed requests (including failed ones)           */
    long long queries;        /* queries of the requests that succeeded               */
    long long batches;        /* device batches run                                   */
    long long failed;         /* requests that ended with an error                    */
    double wall_s;            /* first submission to last completion                  */
    double qps;               /* queries / wall_s                                     */
    double p50_ms, p99_ms;    /* request latency (submission to completion)           */
    double mean_ms, max_ms;
    int max_in_flight;        /* most batches on the device at once                   */
    int slots;
    long long peak_device_bytes;  /* most device bytes held by the slots              */
    long long budget_bytes;
} culsh_server_stats;

int culsh_server_create(culsh_server** out, culsh_index* ix, const culsh_server_config* cfg);
/* Queues Q queries (D x Q column-major host floats, as search()); results go
 * to out_ids / out_dists (K x Q each, as getKnnIds / getKnnDistances). All
 * three buffers must stay valid until culsh_server_wait reports completion. */
int culsh_server_submit(culsh_server* srv, const float* queries, int Q, int K, int T, int* out_ids,
                        float* out_dists, unsigned long long* ticket);
/* Waits up to timeout_s seconds (< 0: no limit). Returns the request's status
 * (its error message in culsh_last_error), or CULSH_PENDING on time-out; a
 * completed ticket is forgotten after it is reported. */
int culsh_server_wait(culsh_server* srv, unsigned long long ticket, double timeout_s);
int culsh_server_stats_get(culsh_server* srv, culsh_server_stats* out);
int culsh_server_stats_reset(culsh_server* srv);
/* Completes every submitted request, then frees the server. */
void culsh_server_destroy(culsh_server* srv);

#ifdef __cplusplus
}
#endif

#endif /* CULSH_C_ABI_H */
