// Internal declarations shared by the CUDA translation units of libculsh.
//
// Device data model of one index (all tables stacked, one allocation each):
//   X        [N][D]  f32    dataset, point-contiguous (the reference's D x N column-major)
//   A        [L*M][D] f32   projection columns; column (l,m) = A[l][m*D .. m*D+D)
//   b        [L*M]   f32
//   cmin/cmax[L*M]   i32    per (table, column) code range
//   fbits/foff[L*M]         bit width / bit offset of each column's field in the packed key
//   ids      [L][N]  u32    point ids sorted by (code row, id): the reference's totalIndices
//   boff     [L+1]   u64    bucket offsets: buckets of table l are [boff[l], boff[l+1])
//   starts/sizes [sum B]    bucket start (within the table's ids) and size
//   ukeys    [sum B][KW]    packed key of each bucket (column 0 in the most significant bits)
//   hslots   [sum H]  u64   bucketized open-addressing hash in 32-byte groups (one
//                           DRAM sector, kGroupWords u64): word 0 holds four 16-bit
//                           fingerprints (0xFFFF = empty), words 1-2 the four 32-bit
//                           bucket indices; probing visits a group's slots in order,
//                           then the next group
//   hoff     [L+1]   u64    word offsets of each table's groups
//   hmask    [L]     u32    power-of-two group count - 1
#pragma once

#include <atomic>
#include <cstdint>
#include <mutex>
#include <cuda_runtime.h>

struct culsh_index;

namespace culsh {

// Makes an index and its dataset device-resident (capi.cu).
int index_make_resident(culsh_index* ix);

constexpr int kMaxM = 64;     // projection columns per table
constexpr int kMaxKW = 8;     // packed key words (256 bits)
constexpr int kMaxT = 256;    // probes per table
constexpr int kMaxK = 2048;   // neighbours per query
constexpr unsigned long long kEmptySlot = ~0ull;
constexpr int kGroupSlots = 4;   // hash slots per 32-byte group
constexpr int kGroupWords = 4;   // u64 words per group
constexpr uint32_t kEmptyFp = 0xFFFFu;

// 16-bit slot fingerprint from the top bits of a key hash (never the empty mark).
__host__ __device__ __forceinline__ uint32_t slot_fp(uint64_t hh) {
    const uint32_t f = (uint32_t)(hh >> 48);
    return f == kEmptyFp ? kEmptyFp - 1 : f;
}

// Device error flags (bit values OR-ed into an int in device memory).
enum DevErr : int {
    kErrNonFinite = 1,     // projection produced NaN/Inf
    kErrCodeRange = 2,     // |code| >= 2^31
    kErrSpin = 4,          // a bounded wait gave up
    kErrHashFull = 8,      // hash insert ran out of probes
    kErrNotIntegral = 16,  // a loaded bucket code is not an integer
};

// splitmix64 finalizer (Steele, Lea, Flood, OOPSLA 2014; public domain).
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__host__ __device__ __forceinline__ uint32_t mix32(uint32_t h) { return (uint32_t)mix64(h); }

constexpr uint64_t kHashSeed = 0x2545f4914f6cdd1dull;

// Lookup hash of a bucket key, additive in its fields: h = sum_m f_m * R_c
// (mod 2^64) over the fields f_m = code_m - cmin_m of table l, with R_c an
// odd 64-bit multiplier per column c = l * M + m, then one mix. A multiprobe
// key differs from its home key by +-1 in some fields, so its hash is the
// home sum +- R_c before the mix. Equal keys hash equally; a lookup verifies
// the stored key on every fingerprint match, so collisions cost time only.
__host__ __device__ __forceinline__ uint64_t field_mult(int c) {
    return mix64(kHashSeed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(c + 1))) | 1ull;
}
__host__ __device__ __forceinline__ uint64_t hash_finish(uint64_t h) { return mix64(h ^ kHashSeed); }

// Key filter beside each table's hash (a blocked Bloom filter, two bits in
// one 32-bit word, 8 to 16 bits per key): the word index and the two bits
// come from the high half of a 64-bit product of the finished hash, so they
// are independent of the group (low bits) and the fingerprint (top 16 bits).
// A key that is in the table always finds both of its bits set.
__host__ __device__ __forceinline__ uint32_t filter_mix(uint64_t hh) {
    return (uint32_t)((hh * 0xD6E8FEB86659FD93ull) >> 32);
}
__host__ __device__ __forceinline__ uint32_t filter_bits(uint32_t fx) {
    return (1u << (fx >> 27)) | (1u << ((fx >> 22) & 31u));
}
constexpr int kFilterBitsPerKey = 8;

// Place a field of `bits` bits (<= 32) at bit offset `off` of a little-endian
// multi-word key.
__host__ __device__ __forceinline__ void key_put(uint32_t* key, int off, int bits, uint32_t val) {
    const int w = off >> 5, s = off & 31;
    key[w] |= val << s;
    if (s != 0 && s + bits > 32) key[w + 1] |= val >> (32 - s);
}

__host__ __device__ __forceinline__ uint32_t key_get(const uint32_t* key, int off, int bits) {
    if (bits == 0) return 0;
    const int w = off >> 5, s = off & 31;
    uint64_t v = key[w] >> s;
    if (s != 0 && s + bits > 32) v |= (uint64_t)key[w + 1] << (32 - s);
    return bits == 32 ? (uint32_t)v : (uint32_t)(v & ((1ull << bits) - 1));
}

// Per-table key layout and lookup structures (device pointers).
struct LookupView {
    int L, M, KW;
    const int32_t* cmin;
    const int32_t* cmax;
    const uint8_t* fbits;
    const uint16_t* foff;
    const uint64_t* boff;
    const uint32_t* starts;
    const uint32_t* sizes;
    const uint32_t* ukeys;
    const unsigned long long* hslots;
    const uint64_t* hoff;
    const uint32_t* hmask;
    const unsigned long long* funit;   // [L*M][2]: 2^foff as (low, high) 64-bit words
    const unsigned long long* rmul;    // [L*M]: field multipliers of the lookup hash
    const uint32_t* filt;              // key filters, table l at words [fl_off[l], fl_off[l+1])
    const uint64_t* fl_off;
    const uint32_t* fl_mask;           // [L]: words in table l's filter - 1 (a power of two - 1)
};

// ---------------------------------------------------------------------------
// Launchers (each returns cudaGetLastError() after the launch).

// Canonical FP32 projection of n_pts points onto the LM stacked columns.
// codes != nullptr: floored codes [LM][n_pts] + per-block min/max partials
// [grid_x][LM]; vals != nullptr: unfloored values [LM][n_pts].
// tile picks the query-value tiling (0: 64x128, 1: 32x128, 2: 128x64 points x columns).
// Word arrays a kernel zeroes on the way (grid-stride, every block takes
// part): the search's first kernel clears the counters the later ones
// accumulate into, instead of two memset nodes in the graph.
struct ZeroWords {
    unsigned long long* a = nullptr;
    int64_t na = 0;
    unsigned long long* b = nullptr;
    int64_t nb = 0;
    __device__ __forceinline__ void clear(int tid) const {
        if (!na && !nb) return;
        const int64_t nthreads = (int64_t)gridDim.x * gridDim.y * blockDim.x;
        const int64_t g = ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * blockDim.x + tid;
        for (int64_t i = g; i < na; i += nthreads) a[i] = 0ull;
        for (int64_t i = g; i < nb; i += nthreads) b[i] = 0ull;
    }
};

// AT: the projection matrix transposed, D rows of lmp floats (lmp = LM rounded
// up to a multiple of 4, columns past LM zero, 16-byte aligned).
cudaError_t launch_project_fp32(const float* X, int64_t n_pts, int D, const float* AT, int lmp, const float* b,
                                int LM, float W, int32_t* codes, float* vals, int32_t* pmin, int32_t* pmax, int* err,
                                cudaStream_t st, int tile = 0, ZeroWords zw = ZeroWords{}, float* xcopy = nullptr);
int project_grid_x(int64_t n_pts);
// The kernel of tiling 5 (xcopy form), for finding its node in a captured
// graph, and its number of parameters (the first is the rows it reads).
const void* project_copy_kernel();
constexpr int kProjectArgs = 15;
// n floats, 16-byte aligned source and destination (src may be host memory
// the device reads directly).
cudaError_t launch_copy_f32(const float* src, float* dst, int64_t n, cudaStream_t st);
cudaError_t launch_minmax_reduce(const int32_t* pmin, const int32_t* pmax, int nparts, int LM, int32_t* cmin,
                                 int32_t* cmax, cudaStream_t st);

// Tensor-core (tcgen05) projection for index builds: plan, bf16 split of X,
// the GEMM with the proven-code epilogue, and the canonical recomputation of
// the codes its error bound could not prove.
struct TcPlan {
    bool ok;
    int Dp, LMp, ntiles, grid, tmem_cols;
    uint32_t b_bytes, x_bytes;
    int stages[2];        // X-tile ring depth without / with the low bf16 part
    size_t smem[2];
};
TcPlan tc_plan(int64_t N, int D, int LM, int num_sms, int max_smem);
// Streaming form for projections whose matrix does not fit shared memory:
// column blocks of blk[need_lo] per launch, any Dp.
struct TcStreamPlan {
    bool ok;
    int Dp, LMp, ntiles, grid;
    int blk[2], stages[2];
    size_t smem[2];
};
TcStreamPlan tc_plan_stream(int64_t N, int D, int LM, int num_sms, int max_smem);
cudaError_t launch_project_tc_stream(const TcStreamPlan& p, int need_lo, int64_t N, int D, int LM, const void* xh,
                                     const void* xl, const void* ah, const void* al, const float* b,
                                     const float* anorm, const float* xnorm, float W, float kappa, int32_t* codes,
                                     int32_t* pmin, int32_t* pmax, unsigned long long* relist,
                                     unsigned long long relist_cap, unsigned int* relist_cnt, int* err,
                                     cudaStream_t st);
cudaError_t launch_split_rows(const float* X, int64_t N, int D, int Dp, void* xh, void* xl, float* xnorm, int* flags,
                              cudaStream_t st);
cudaError_t launch_project_tc(const TcPlan& p, int need_lo, int64_t N, int D, int LM, const void* xh, const void* xl,
                              const void* ah, const void* al, const float* b, const float* anorm, const float* xnorm,
                              float W, float kappa, int32_t* codes, int32_t* pmin, int32_t* pmax,
                              unsigned long long* relist, unsigned long long relist_cap, unsigned int* relist_cnt,
                              int* err, cudaStream_t st);
cudaError_t launch_tc_recompute(const float* X, int64_t N, int D, int LM, const float* A, const float* b, float W,
                                const unsigned long long* list, unsigned long long cap, const unsigned int* cnt,
                                int regions, int32_t* codes, int32_t* cmin, int32_t* cmax, int* err, cudaStream_t st);

// Key packing from int codes [LM][N] into SoA keys [KW][L*N] and identity values.
cudaError_t launch_pack_keys(const int32_t* codes, int64_t N, int L, int M, int KW, const int32_t* cmin,
                             const uint8_t* fbits, const uint16_t* foff, uint32_t* keys, uint32_t* vals,
                             cudaStream_t st);

// Onesweep segmented LSD radix sort of L segments of N (key, value) pairs.
// Sorts bits [0, 8*passes) of the KW-word keys. Buffers are ping-ponged; on
// return *result_in_alt tells whether the sorted data sits in the alt buffers.
struct SortBuffers {
    uint32_t* keys[2];   // [KW][L*N] each
    uint32_t* vals[2];   // [L*N] each
    uint32_t* hist;      // [L][passes][256]
    uint32_t* base;      // [L][passes][256]
    uint32_t* status;    // [L*tiles][256] + counter
    int* err;
    uint32_t* h_hist = nullptr;   // pinned host copy of hist (allocated per call when absent or short)
    size_t h_hist_words = 0;
};
size_t sort_status_words(int64_t N, int L);
cudaError_t run_segmented_sort(SortBuffers& sb, int64_t N, int L, int KW, int passes, bool* result_in_alt,
                               cudaStream_t st);

// Top-word-first ordering (sort.cu): after the digit passes over the top key
// word, gather the lower words into sorted order, find the runs of equal top
// words and order each run by (lower words, id).
struct RunLists {
    unsigned long long* tpos;   // runs of 2..8: first sorted position (table * N + i)
    uint32_t* tlen;
    unsigned int tcap;
    unsigned long long* spos;   // runs of 9..32
    uint32_t* slen;
    unsigned int scap;
    unsigned long long* lpos;   // runs of 33..run_max_len()
    uint32_t* llen;
    unsigned int lcap;
    unsigned int* cnt;          // [4]: tiny, small and large runs; overflow flags (1 run too long, 2 list full)
};
cudaError_t launch_gather_lower(const uint32_t* keys0, const uint32_t* ids, const uint32_t* top, int64_t N, int L,
                                int KW, uint32_t* skeys, cudaStream_t st);
cudaError_t launch_run_find(const uint32_t* top, int64_t N, int L, const RunLists& rl, cudaStream_t st);
cudaError_t launch_run_sorts(const RunLists& rl, const unsigned int* counts, int64_t N, int L, int KW, uint32_t* skeys,
                             uint32_t* ids, cudaStream_t st);
int run_max_len();

// Run-length bucketing of sorted keys. Two phases: count (per table bucket
// totals, written to nb[L]) and write (starts, ukeys).
cudaError_t launch_rl_count(const uint32_t* keys, int64_t N, int L, int KW, uint32_t* tile_cnt, uint32_t* tile_off,
                            uint32_t* nb, cudaStream_t st);
cudaError_t launch_rl_write(const uint32_t* keys, int64_t N, int L, int KW, const uint32_t* tile_off,
                            const uint64_t* boff, uint32_t* starts, uint32_t* ukeys, cudaStream_t st);
cudaError_t launch_bucket_sizes(const uint64_t* boff, const uint32_t* starts, int64_t N, int L, int64_t maxB,
                                uint32_t* sizes, uint32_t* max_size, cudaStream_t st);
cudaError_t launch_hash_build(const uint64_t* boff, const uint32_t* ukeys, int L, int M, int KW, int64_t maxB,
                              const uint16_t* foff, const uint8_t* fbits, const unsigned long long* rmul,
                              const uint64_t* hoff, const uint32_t* hmask, unsigned long long* hslots,
                              uint32_t* filt, const uint64_t* fl_off, const uint32_t* fl_mask, int* err,
                              cudaStream_t st);
// Bucket codes [M][B_l] per table (float, the reference's layout) decoded from ukeys.
cudaError_t launch_decode_codes(const uint64_t* boff, const uint32_t* ukeys, int L, int M, int KW, int64_t maxB,
                                const int32_t* cmin, const uint8_t* fbits, const uint16_t* foff, float* codes,
                                cudaStream_t st);
// From loaded float bucket codes: per (l,m) min/max + integrality check, then ukeys.
cudaError_t launch_codes_minmax(const uint64_t* boff, const float* codes, int L, int M, int64_t maxB,
                                int32_t* cmin, int32_t* cmax, int* err, cudaStream_t st);
cudaError_t launch_pack_from_codes(const uint64_t* boff, const float* codes, int L, int M, int KW, int64_t maxB,
                                   const int32_t* cmin, const uint8_t* fbits, const uint16_t* foff, uint32_t* ukeys,
                                   cudaStream_t st);

// Random projection (seeded counter-based generator): A ~ N(0,1), u ~ U(0,1].
cudaError_t launch_random_projection(float* A, float* u, int64_t nA, int64_t nu, unsigned long long seed,
                                     cudaStream_t st);

// Query side.
struct ProbeArgs {
    const float* vals;         // [L*M][Q] unfloored projections
    int Q, T;
    LookupView lv;
    int32_t* qbuckets;         // [L][Q*T]
    unsigned long long* cnu;   // [Q] non-unique candidate counts (accumulated)
    int small_codes;           // every |cmin|, |cmax| < 2^24 - 2 (set by the host)
    int pch;                   // fast kernel: probes whose group loads overlap (1, 2, 4)
    // Split lookups (M <= 16, fast kernel). split = 1: the enumeration kernel
    // stores each valid probe's finished hash and mask and marks its query
    // bucket -2; k_probe_resolve then checks the key filter and walks the
    // hash. split = 2: the enumeration kernel stores them and looks its
    // pair's probes up itself, behind the filter, at its end.
    int split;
    unsigned long long* ph;    // [L][T][Q] finished hash of each pending probe
    uint32_t* pmask;           // [L][T][Q] its mask over the sorted deltas
    uint4* pctx;               // [L*Q][3] home key (128 bits), sorted deltas (32 bytes)
};
cudaError_t launch_probe(const ProbeArgs& a, cudaStream_t st);
int probe_launches(const ProbeArgs& a);   // kernels launch_probe launches

struct CandArgs {
    const float* X;
    int64_t N;
    int D, L, T, Q, K;
    const float* queries;              // [Q][D]
    const int32_t* qbuckets;           // [L][Q*T]
    const uint64_t* boff;
    const uint32_t* starts;
    const uint32_t* sizes;
    const uint32_t* ids;               // [L][N]
    const unsigned long long* cnu;     // [Q]
    int32_t* out_ids;                  // [Q][K]
    float* out_d;                      // [Q][K]
    unsigned long long* cu;            // [Q] unique counts
    unsigned long long* totals;        // [2]: sum unique, sum non-unique
    uint32_t* arena;                   // overflow hash sets for large candidate sets
    unsigned long long arena_words;
    unsigned long long* arena_top;
    int* deferred;                     // [Q] list of queries that did not fit the arena
    unsigned int* n_deferred;
    const int* qlist;                  // optional subset of queries (nullptr = all)
    int nq;
};
// Work-stealing form of the candidate stage (candidates.cu): queries split
// into id-partition items, claimed by a persistent grid.
struct WsArgs {
    const float* X;
    int64_t N;
    int D, L, T, Q, K;
    const float* queries;              // [Q][D]
    const int32_t* qbuckets;           // [L][Q*T]
    const uint64_t* boff;
    const uint32_t* starts;
    const uint32_t* sizes;
    const uint32_t* ids;               // [L][N]
    const unsigned long long* cnu;     // [Q]
    int32_t* out_ids;                  // [Q][K]
    float* out_d;                      // [Q][K]
    unsigned long long* cu;            // [Q] unique counts
    unsigned long long* totals;        // [2]: sum unique, sum non-unique
    int pmax;                          // partitions per query, at most 64
    unsigned long long chunk;          // non-unique candidates per partition
    int* q_items;                      // [Q] partitions of each query
    int* q_off;                        // [Q] first item of each query
    unsigned int* q_done;              // [Q] partitions finished
    int* item_q;                       // [item_cap]
    uint8_t* item_p;                   // [item_cap]
    int* part_n;                       // [item_cap] partial list lengths
    float* part_d;                     // [item_cap][K]
    uint32_t* part_i;                  // [item_cap][K]
    unsigned int item_cap;
    unsigned int* n_items;
    unsigned int* next_item;           // work-stealing counter, zero before the launch
    unsigned int* overflow;            // nonzero: rerun with the per-query kernel
    int wt;                            // threads per item CTA: 64, 128 or 256
    int slots;                         // shared hash-set slots per item: 4096 or 8192
    // BF16 form: approximate distances from xb, certified FP32 rerank
    int bf16;
    const uint16_t* xb;                // [N][D] bf16 copy of X
    const uint8_t* xflag;              // [N] 1 exact in bf16, 2 always re-check, 0 bound applies
    float e_c1, e_c2;                  // error-bound factors (rounded up)
    unsigned long long* rechecked;     // candidates whose FP32 row pass 2 re-read
    // Dense form: queries with at least dense_min non-unique candidates
    unsigned long long dense_min;      // ~0ull: never
    int* dense_q;                      // [Q] queries routed to the bitmap kernel
    unsigned int* n_dense;
    unsigned int* dense_next;          // claim counter of the bitmap kernel
    // Locality order (tuned): queries planned in the order of their home
    // bucket in table 0 (launch_order_queries), so that items of queries
    // with shared candidates run close together and share rows in L2.
    uint32_t* order;                   // [Q] queries in that order; nullptr: index order
    uint32_t* order_bins;              // [kOrderBins + 1] counting-sort bins
    // Bucket rows (tensor-core path): the index's largest buckets as N-bit
    // rows, ORed into a dense query's membership row instead of setting the
    // bits of their ids one by one. big_gi holds their global bucket numbers
    // (boff[l] + j) in ascending order; every bucket of big_min ids or more
    // has a row. nbig == 0: none.
    const uint64_t* big_gi;
    const uint32_t* big_rows;          // [nbig][nwp]
    int nbig;
    uint32_t big_min;
};
constexpr int kOrderBins = 4096;
cudaError_t launch_order_queries(const WsArgs& a, cudaStream_t st);   // 3 kernels + 1 memset
size_t dense_smem_bytes(int64_t N, int D, int K);
cudaError_t launch_candidates_dense(const WsArgs& a, int grid, cudaStream_t st);
size_t ws_smem_bytes(int D, int K, int wt, int bf16, int slots);
int ws_blocks_per_sm(int D, int K, int wt, int bf16, int slots);
cudaError_t launch_bf16_rows(const float* X, int64_t N, int D, uint16_t* xb, uint8_t* flag, cudaStream_t st);
cudaError_t launch_plan_items(const WsArgs& a, cudaStream_t st);
// Bucket rows: the global numbers and sizes of the buckets of at least
// big_min ids (at most cap, in no order; *cnt counts them), then their rows
// (rows zeroed beforehand; tl[r] is bucket r's table).
cudaError_t launch_big_find(const uint32_t* sizes, uint64_t totB, uint32_t big_min, uint64_t* gi, uint32_t* sz,
                            unsigned int* cnt, unsigned int cap, cudaStream_t st);
cudaError_t launch_big_fill(const uint64_t* gi, const int32_t* tl, int nbig, const uint32_t* starts,
                            const uint32_t* sizes, const uint32_t* ids, int64_t N, uint32_t* rows, int nwp,
                            cudaStream_t st);
cudaError_t launch_candidates_ws(const WsArgs& a, int grid, cudaStream_t st);

// ---------------------------------------------------------------------------
// Tensor-core k-NN over candidate membership rows (knn_tc.cu): the dense
// queries' candidate distances and top-K as a masked GEMM.

// Properties of a set of rows (the dataset, or one search's dense queries),
// accumulated by k_knn_rows. Zero is the empty state.
enum KnnFlags : int {
    kKnnHasLo = 1,         // some value is not exact in bf16
    kKnnNotSmallInt = 2,   // some value is not an integer of magnitude <= 256
    kKnnNonFinite = 4,
};
struct KnnState {
    int flags;
    int mneg;   // max over the small-integer values v of 257 - v (0: none)
    int mpos;   // max over them of v + 257
    int pad;
};
constexpr int kMaxKnnK = 64;    // list length limit of the tensor-core k-NN path
constexpr int kKnnTileQ = 128;  // queries per tensor-core tile

// Everything the k-NN kernels of one search read and write.
struct KnnSearch {
    int N, D, Dp, K, Qcap;            // Qcap: rows of the query buffers (a multiple of 128)
    int grid;                          // persistent CTAs of the tensor-core kernels
    int exact_possible;                // dataset qualifies for the exact form (launch its kernel)
    int kl_exact, kl_bound;            // list length per query (exact: K; bound: K + margin)
    int ops_exact, ops_bound;          // point-tile ring stages per form
    size_t smem_exact, smem_bound;     // dynamic shared memory per form
    int nwp;                           // membership words per query row (a multiple of 4)
    float C;                           // bound-form factor (|d~ - d| <= C S)
    // dataset side (per index)
    const void* xh;                    // [N][Dp] bf16
    const void* xl;                    // [N][Dp] bf16
    const float* w_exact;              // [ntp256 * 256]: |x|^2, FLT_MAX past N
    const float* w_bound;              // [ntp256 * 256]: |x|^2 - C |x|^2_up, FLT_MAX past N
    const KnnState* dstate;
    const float* X;                    // [N][D] f32 (the bound form's exact recomputation)
    // query side (per search)
    const float* queries;              // [Q][D] f32
    const int* dense_q;                // dense list (query ids)
    const unsigned int* n_dense;
    void* qh;                          // [Qcap][Dp] bf16, dense-list order
    void* ql;
    float* qsq;                        // [Qcap]
    float* qbase;                      // [Qcap]
    KnnState* qstate;                  // cleared before the search
    unsigned int* qbound;              // [Qcap] exact form: per-query shared key bound
    const uint32_t* bm;                // [Qcap][nwp] membership rows (k_cand_bitmap)
    float* part_key;                   // partial lists, see k_knn_tc
    uint32_t* part_id;
    int* part_n;
    int32_t* out_ids;
    float* out_d;
    int* fallback;                     // [Qcap] queries the bound form could not prove
    unsigned int* n_fallback;
    int* err;
};
// Buffer sizes of one search (elements).
size_t knn_part_entries(const KnnSearch& k);   // part_key / part_id entries
size_t knn_part_lists(const KnnSearch& k);     // part_n entries
// Plans the shared memory and stages of both forms for D, K on this device;
// false when the tensor-core path cannot serve them (D > 128, K too large).
bool knn_plan(KnnSearch& k, int max_smem);
// The bound-form factor C for dimension D (see knn_tc.cu).
float knn_bound_factor(int D);
// Dataset rows: bf16 parts, weights, flags (once per index).
cudaError_t launch_knn_rows_dataset(const float* X, int64_t N, int D, int Dp, void* xh, void* xl, float* w_exact,
                                    float* w_bound, int64_t pad, float C, KnnState* st, cudaStream_t s);
// Query rows, tensor-core kernels and merge of one search (3 or 4 launches).
cudaError_t launch_knn_search(const KnnSearch& k, cudaStream_t s);
int knn_launches(const KnnSearch& k);
// Membership rows of the dense queries (candidates.cu).
size_t bitmap_smem_bytes(int64_t N);
cudaError_t launch_cand_bitmap(const WsArgs& a, uint32_t* bm, int nwp, int grid, cudaStream_t st);

// Opts `func` into `dyn` bytes of dynamic shared memory when static plus
// dynamic shared memory could pass the 48 KB default (the kernels here keep
// at most 12 KB static). The opted-in size only grows (`cap` records it per
// kernel), so a smaller configuration launched later stays valid.
template <class F>
cudaError_t opt_in_smem(F* func, size_t dyn, std::atomic<size_t>& cap) {
    if (dyn + 12 * 1024 <= 48 * 1024 || dyn <= cap.load()) return cudaSuccess;
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    if (dyn <= cap.load()) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e == cudaSuccess) cap = dyn;
    return e;
}

// Process-wide lock held while a search plans (and grows) its buffers and
// captures its graph: no thread frees device memory while another captures.
std::mutex& alloc_capture_mutex();
// Sets the calling thread's culsh_last_error() message; returns code.
int set_last_error(int code, const char* msg);

int cand_smem_capacity();              // candidates handled in shared memory per query
cudaError_t launch_candidates(const CandArgs& a, cudaStream_t st);
size_t cand_arena_words(unsigned long long nonunique);

}  // namespace culsh
