// Host orchestration and C ABI of libculsh.
//
// Mirrors the state and call sequence of cuLSH::HashTables
// (cuLSH_HashTables.cu) and cuLSH::SearchTables (cuLSH_SearchTables.cu), with
// the data kept resident on one GPU: index() uploads the dataset once and
// builds all tables together, each stage one pass over every table
// (projection with exact codes, key packing, one radix sort over all tables,
// run-length encoding, bucket hash and key filters), and search() replays the
// whole query path (projection, multiprobe, candidate stage: four to nine
// kernels) as one captured CUDA graph. Host copies of the bucket arrays and
// query buckets are produced lazily, only when a getter or save() needs them.
#include <algorithm>
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <mutex>
#include <string>
#include <vector>

#include "culsh.h"
#include "culsh_internal.cuh"

using namespace culsh;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CU_TRY(call)                                                                                   \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            return fail(e_ == cudaErrorMemoryAllocation ? CULSH_ERR_OUT_OF_MEMORY : CULSH_ERR_CUDA,    \
                        "%s: %s", #call, cudaGetErrorString(e_));                                      \
    } while (0)

#define TRY(expr)                  \
    do {                           \
        int rc_ = (expr);          \
        if (rc_ != CULSH_OK) return rc_; \
    } while (0)

template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t reserve(size_t cnt) {
        if (cnt <= n && p) return cudaSuccess;
        release();
        const cudaError_t e = cudaMalloc(&p, std::max<size_t>(cnt, 1) * sizeof(T));
        if (e == cudaSuccess) n = std::max<size_t>(cnt, 1);
        else p = nullptr;
        return e;
    }
    void swap(DevBuf& o) {
        std::swap(p, o.p);
        std::swap(n, o.n);
    }
};

template <class T>
struct PinBuf {
    T* p = nullptr;
    size_t n = 0;
    PinBuf() = default;
    PinBuf(const PinBuf&) = delete;
    PinBuf& operator=(const PinBuf&) = delete;
    ~PinBuf() {
        if (p) cudaFreeHost(p);
    }
    cudaError_t reserve(size_t cnt) {
        if (cnt <= n && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        const cudaError_t e = cudaMallocHost(&p, std::max<size_t>(cnt, 1) * sizeof(T));
        if (e == cudaSuccess) n = std::max<size_t>(cnt, 1);
        return e;
    }
};

inline uint64_t next_pow2(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

inline double seconds_now() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

}  // namespace

struct culsh_index {
    int N = 0, D = 0, L = 0, M = 0;
    float W = 0.0f;
    std::vector<float> A, b;   // [L][M][D] (A[l] column-major D x M), [L][M]
    bool has_proj = false;

    // index state
    bool indexed = false, host_valid = false, dev_valid = false;
    std::vector<uint32_t> buckets;   // [L]
    std::vector<std::vector<uint32_t>> h_ids, h_starts, h_sizes;
    std::vector<std::vector<float>> h_codes;

    // device
    cudaStream_t stream = nullptr;
    DevBuf<float> X;               // owned dataset copy
    const float* x_src = nullptr;  // host pointer the copy was made from
    const float* x_borrow = nullptr;
    DevBuf<float> dA, db;
    DevBuf<float> dAT;           // A transposed: D rows of lmp floats, columns past L*M zero
    std::vector<float> at_host;  // host staging of dAT (kept alive for the asynchronous copy)
    int lmp = 0;                 // L*M rounded up to a multiple of 4
    bool proj_on_dev = false;
    DevBuf<uint16_t> xb;    // bf16 copy of the device dataset (search precision form), built on first use
    DevBuf<uint8_t> xflag;  // per row: 1 exact in bf16, 2 always re-check in FP32, 0 bound applies
    bool xb_valid = false;
    // tensor-core k-NN rows of the dataset (bf16 parts, weights, flags), built on first use
    DevBuf<uint16_t> kx_h, kx_l;
    DevBuf<float> kw_exact, kw_bound;
    DevBuf<KnnState> kstate;
    KnnState h_kstate{};
    bool kx_valid = false;
    // bucket rows of the largest buckets (membership rows of the tensor-core
    // path), made on first use after each build or load
    DevBuf<uint64_t> big_gi;
    DevBuf<int32_t> big_tl;
    DevBuf<uint32_t> big_sz, big_rows;
    DevBuf<unsigned int> big_cnt;
    int nbig = 0;
    uint32_t big_min = UINT32_MAX;
    bool big_valid = false;
    int KW = 1;
    std::vector<int32_t> h_cmin, h_cmax;
    std::vector<uint8_t> h_fbits;
    std::vector<uint16_t> h_foff;
    DevBuf<int32_t> cmin, cmax;
    DevBuf<uint8_t> fbits;
    DevBuf<uint16_t> foff;
    DevBuf<unsigned long long> funit;   // [L*M][2]: 2^foff as two 64-bit words
    DevBuf<unsigned long long> rmul;    // [L*M]: lookup-hash field multipliers
    DevBuf<uint32_t> ids, starts, sizes, ukeys;
    std::vector<uint64_t> h_boff, h_hoff;
    std::vector<uint32_t> h_hmask;
    DevBuf<uint64_t> boff, hoff;
    DevBuf<uint32_t> hmask;
    DevBuf<unsigned long long> hslots;
    std::vector<uint64_t> h_fl_off;   // key filters (see filter_mix)
    std::vector<uint32_t> h_fl_mask;
    DevBuf<uint64_t> fl_off;
    DevBuf<uint32_t> fl_mask, filt;
    DevBuf<float> dcodes;
    DevBuf<int> err;

    // build workspace (kept across builds)
    DevBuf<int32_t> ws_codes, ws_pmin, ws_pmax;
    DevBuf<uint16_t> ws_ah, ws_al, ws_xh, ws_xl;   // bf16 splits for the tensor-core projection
    DevBuf<float> ws_anorm, ws_xnorm;
    DevBuf<int> ws_tcflags;
    double tc_predicted_open = 0.0;   // predicted share of codes the tensor-core bound leaves open
    DevBuf<uint32_t> maxb;
    PinBuf<uint32_t> h_maxb;
    uint32_t max_bucket = 0;          // largest bucket of any table (gates the dense candidate kernel)
    DevBuf<unsigned long long> ws_relist;
    DevBuf<unsigned int> ws_relist_cnt;
    long long tc_recomputed = -1;   // codes recomputed after the tensor-core pass (-1: SIMT path)
    int tc_need_lo = 0;
    int sort_passes = 0;
    cudaEvent_t bev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};   // build stage boundaries
    bool built_once = false;
    DevBuf<uint32_t> ws_keys[2], ws_vals, ws_hist, ws_base, ws_status, ws_tcnt, ws_toff, ws_nb;
    PinBuf<uint32_t> h_sort_hist;
    DevBuf<unsigned long long> ws_run_pos;
    DevBuf<uint32_t> ws_run_len;
    DevBuf<unsigned int> ws_run_cnt;
    PinBuf<unsigned int> h_run_cnt;
    int sort_form = 0;   // 1: top-word passes + run ordering, 2: that form fell back to all words, 0: all words

    ~culsh_index() {
        for (auto& e : bev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
    const float* dev_x() const { return x_borrow ? x_borrow : (X.p ? X.p : nullptr); }
};

// Tuning knobs of the search path (culsh_search_autotune picks them).
struct SearchTune {
    int proj_tile = 0;     // query projection tiling (launch_project_fp32)
    int probe_pch = 2;     // probes whose hash-group loads overlap (1, 2, 4)
    int cand_ws = 1;       // 1: work-stealing candidate kernel, 0: one block per query
    int ws_wt = 128;       // threads per work item (64, 128, 256, 512)
    int ws_bps = 0;        // resident work-stealing CTAs per SM (0: occupancy limit)
    int ws_chunk = 1024;   // non-unique candidates per id partition
    int dist_bf16 = 0;     // 1: BF16 candidate distances + certified FP32 rerank (work-stealing form)
    int ws_slots = 4096;   // shared hash-set slots per work item (4096, 8192 or 16384)
    int probe_split = 0;   // M <= 16: 1 enumeration kernel + lookup kernel; 2 lookups at the enumeration's end
    int ws_order = 0;      // 1: plan queries in the locality order of their home bucket (work-stealing form)
    int dense_tc = 1;      // 1: dense queries take the tensor-core path (membership rows + masked GEMM)
    int dense_min = 0;     // non-unique candidates that make a query dense (0: the form's default)
};
constexpr size_t kPlanBytes = 2048;   // room for the graph key (checked below)

struct culsh_search {
    culsh_index* ix = nullptr;
    int K = 0, T = 1, Q = 0, L = 0;
    bool searched = false;
    unsigned long long tot_unique = 0, tot_nonunique = 0;
    culsh_times times{};
    cudaStream_t stream = nullptr;
    // stage boundaries: [0..3] search stages, [4] host copy done, [5] membership rows done
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int launches = 0, deferred_queries = 0;
    bool host_copy_timed = false;
    DevBuf<float> dq, vals, od;
    DevBuf<int32_t> qb, oids;
    DevBuf<unsigned long long> ph;   // split probe lookups: hash, mask, pair context
    DevBuf<uint32_t> pmask;
    DevBuf<uint4> pctx;
    DevBuf<unsigned long long> cnu, cu, stats;
    DevBuf<int> deferred;
    DevBuf<uint32_t> arena;
    // work-stealing candidate stage
    DevBuf<int> q_items, q_off, item_q, part_n, dense_q;
    DevBuf<uint32_t> qorder, qorder_bins;
    DevBuf<unsigned int> q_done;
    DevBuf<uint8_t> item_p;
    DevBuf<float> part_d;
    DevBuf<uint32_t> part_i;
    // tensor-core k-NN path: membership rows, query rows, partial lists, fallback list
    DevBuf<uint32_t> kbm;
    DevBuf<uint16_t> kq_h, kq_l;
    DevBuf<float> kq_sq, kq_base, kpart_key;
    DevBuf<unsigned int> kq_bound;
    DevBuf<uint32_t> kpart_id;
    DevBuf<int> kpart_n, kfallback;
    int knn_queries = 0, knn_fallback = 0;   // last search: dense queries on the tensor cores, re-run
    int bucket_rows = 0;                     // last search: bucket rows its membership rows could use
    int sms = 0, smem_optin = 0, ws_used = 0, ws_overflow = 0;
    long long occ_key = -1;
    int occ_val = 1;
    long long rechecked = 0;   // BF16 form: candidates re-read in FP32 by the last search
    int dense_queries = 0;     // queries of the last search that took the bitmap kernel
    int host_path = 0;  // last search: 0 device buffers, 1 staged host copies, 2 direct host access,
                        // 3 direct host access with the copy fused into the projection
    SearchTune tune;
    bool use_graphs = true;
    bool stage_events = true;        // record the four stage events (culsh_search_set_profiling)
    bool last_stage_events = true;   // whether the last search recorded them
    cudaGraphExec_t gexec = nullptr;     // cached search graph and the plan it was captured from
    cudaGraph_t graph = nullptr;         // the captured graph (its projection node is updated in place)
    cudaGraphNode_t gproj = nullptr;     // projection node of the fused host-copy form, if found
    const float* gsrc = nullptr;         // host query rows the instantiated projection node reads
    unsigned char gplan[kPlanBytes] = {};
    int glaunches = 0, graph_mode = 0;
    PinBuf<int32_t> h_ids, h_qb;
    PinBuf<float> h_d;
    PinBuf<unsigned long long> h_stats;
    bool qb_host_valid = false;

    ~culsh_search() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

int ensure_stream(cudaStream_t* st) {
    if (!*st) CU_TRY(cudaStreamCreateWithFlags(st, cudaStreamNonBlocking));
    return CULSH_OK;
}

int check_params(int N, int D, int L, int M, float W) {
    // cuLSH_HashTables.cu:70 checkParameters: all positive.
    if (!(N > 0 && D > 0 && L > 0 && M > 0 && W > 0.0f))
        return fail(CULSH_ERR_INVALID_ARGUMENT,
                    "Projection parameters must be positive! (N, D, L, M, W) = (%d, %d, %d, %d, %g)", N, D, L, M,
                    (double)W);
    if (!std::isfinite(W)) return fail(CULSH_ERR_INVALID_ARGUMENT, "W must be finite");
    if (N > CULSH_MAX_N) return fail(CULSH_ERR_CAPACITY, "N = %d exceeds the supported maximum %d", N, CULSH_MAX_N);
    if (M > CULSH_MAX_M) return fail(CULSH_ERR_CAPACITY, "M = %d exceeds the supported maximum %d", M, CULSH_MAX_M);
    return CULSH_OK;
}

void clear_index_state(culsh_index* ix) {
    ix->indexed = ix->host_valid = ix->dev_valid = false;
    ix->buckets.clear();
    ix->h_ids.clear();
    ix->h_starts.clear();
    ix->h_sizes.clear();
    ix->h_codes.clear();
    ix->x_src = nullptr;
    ix->x_borrow = nullptr;
    ix->proj_on_dev = false;
    ix->xb_valid = false;
    ix->kx_valid = false;
    ix->big_valid = false;
}

int upload_projection(culsh_index* ix, cudaStream_t st) {
    if (ix->proj_on_dev) return CULSH_OK;
    const size_t LM = (size_t)ix->L * ix->M;
    CU_TRY(ix->dA.reserve(LM * ix->D));
    CU_TRY(ix->db.reserve(LM));
    CU_TRY(cudaMemcpyAsync(ix->dA.p, ix->A.data(), sizeof(float) * LM * ix->D, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(ix->db.p, ix->b.data(), sizeof(float) * LM, cudaMemcpyHostToDevice, st));
    const int D = ix->D;
    const int lmp = (int)((LM + 3) & ~(size_t)3);
    ix->at_host.assign((size_t)lmp * D, 0.0f);
    for (size_t c = 0; c < LM; ++c)
        for (int d = 0; d < D; ++d) ix->at_host[(size_t)d * lmp + c] = ix->A[c * D + d];
    CU_TRY(ix->dAT.reserve((size_t)lmp * D));
    CU_TRY(cudaMemcpyAsync(ix->dAT.p, ix->at_host.data(), sizeof(float) * lmp * D, cudaMemcpyHostToDevice, st));
    ix->lmp = lmp;
    ix->proj_on_dev = true;
    return CULSH_OK;
}

int read_err_flag(culsh_index* ix, cudaStream_t st, const char* what) {
    int h = 0;
    CU_TRY(cudaMemcpyAsync(&h, ix->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    if (h & kErrNonFinite) return fail(CULSH_ERR_NUMERIC, "%s: a projection is not finite (NaN/Inf in the data?)", what);
    if (h & kErrCodeRange) return fail(CULSH_ERR_NUMERIC, "%s: a bucket code exceeds the int32 range", what);
    if (h & kErrNotIntegral) return fail(CULSH_ERR_FORMAT, "%s: a bucket code is not an integer", what);
    if (h & kErrSpin) return fail(CULSH_ERR_DEVICE, "%s: a device-side wait gave up", what);
    if (h & kErrHashFull) return fail(CULSH_ERR_DEVICE, "%s: hash table insert ran out of slots", what);
    return CULSH_OK;
}

// Bit widths and offsets of each column's field: column 0 most significant.
int compute_layout(culsh_index* ix, int* passes) {
    const int L = ix->L, M = ix->M;
    ix->h_fbits.assign((size_t)L * M, 0);
    ix->h_foff.assign((size_t)L * M, 0);
    int smax = 0;
    for (int l = 0; l < L; ++l) {
        int off = 0;
        for (int m = M - 1; m >= 0; --m) {
            const int c = l * M + m;
            const int64_t range = (int64_t)ix->h_cmax[c] - (int64_t)ix->h_cmin[c];
            int bits = 0;
            while (bits < 63 && (range >> bits) != 0) ++bits;
            if (bits > 32) return fail(CULSH_ERR_CAPACITY, "code range of table %d column %d needs %d bits", l, m, bits);
            ix->h_fbits[c] = (uint8_t)bits;
            ix->h_foff[c] = (uint16_t)off;
            off += bits;
        }
        smax = std::max(smax, off);
    }
    if (smax > 32 * kMaxKW)
        return fail(CULSH_ERR_CAPACITY, "bucket codes need %d key bits per table, more than the supported %d", smax,
                    32 * kMaxKW);
    ix->KW = std::max(1, (smax + 31) / 32);
    *passes = (smax + 7) / 8;
    return CULSH_OK;
}

int upload_layout(culsh_index* ix, cudaStream_t st) {
    const size_t LM = (size_t)ix->L * ix->M;
    CU_TRY(ix->fbits.reserve(LM));
    CU_TRY(ix->foff.reserve(LM));
    CU_TRY(ix->cmin.reserve(LM));
    CU_TRY(ix->cmax.reserve(LM));
    CU_TRY(cudaMemcpyAsync(ix->fbits.p, ix->h_fbits.data(), LM, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(ix->foff.p, ix->h_foff.data(), LM * 2, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(ix->cmin.p, ix->h_cmin.data(), LM * 4, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(ix->cmax.p, ix->h_cmax.data(), LM * 4, cudaMemcpyHostToDevice, st));
    std::vector<unsigned long long> unit(2 * LM, 0ull);
    for (size_t c = 0; c < LM; ++c) {
        const int off = ix->h_foff[c];
        if (off < 64) unit[2 * c] = 1ull << off;
        else if (off < 128) unit[2 * c + 1] = 1ull << (off - 64);
    }
    CU_TRY(ix->funit.reserve(2 * LM));
    CU_TRY(cudaMemcpyAsync(ix->funit.p, unit.data(), 16 * LM, cudaMemcpyHostToDevice, st));
    std::vector<unsigned long long> rm(LM);
    for (size_t c = 0; c < LM; ++c) rm[c] = field_mult((int)c);
    CU_TRY(ix->rmul.reserve(LM));
    CU_TRY(cudaMemcpyAsync(ix->rmul.p, rm.data(), 8 * LM, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaStreamSynchronize(st));   // `unit` and `rm` are pageable temporaries
    return CULSH_OK;
}

// Hash tables over the unique keys, load factor between 1/4 and 1/2, in
// groups of kGroupSlots slots.
int build_hash(culsh_index* ix, cudaStream_t st) {
    const int L = ix->L;
    ix->h_hoff.assign(L + 1, 0);
    ix->h_hmask.assign(L, 0);
    int64_t maxB = 0;
    for (int l = 0; l < L; ++l) {
        const uint64_t B = ix->h_boff[l + 1] - ix->h_boff[l];
        const uint64_t groups = next_pow2(std::max<uint64_t>(2 * B, kGroupSlots)) / kGroupSlots;
        ix->h_hmask[l] = (uint32_t)(groups - 1);
        ix->h_hoff[l + 1] = ix->h_hoff[l] + groups * kGroupWords;
        maxB = std::max<int64_t>(maxB, (int64_t)B);
    }
    CU_TRY(ix->hoff.reserve(L + 1));
    CU_TRY(ix->hmask.reserve(L));
    CU_TRY(ix->hslots.reserve(ix->h_hoff[L]));
    CU_TRY(cudaMemcpyAsync(ix->hoff.p, ix->h_hoff.data(), 8 * (L + 1), cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(ix->hmask.p, ix->h_hmask.data(), 4 * L, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemsetAsync(ix->hslots.p, 0xFF, 8 * ix->h_hoff[L], st));
    // Filter words per table: a power of two holding 8 to 16 bits per key.
    ix->h_fl_off.assign(L + 1, 0);
    std::vector<uint32_t>& flm = ix->h_fl_mask;
    flm.assign(L, 0);
    for (int l = 0; l < L; ++l) {
        const uint64_t B = ix->h_boff[l + 1] - ix->h_boff[l];
        const uint64_t words = next_pow2(std::max<uint64_t>((B * kFilterBitsPerKey + 31) / 32, 1));
        flm[l] = (uint32_t)(words - 1);
        ix->h_fl_off[l + 1] = ix->h_fl_off[l] + words;
    }
    CU_TRY(ix->fl_off.reserve(L + 1));
    CU_TRY(ix->fl_mask.reserve(L));
    CU_TRY(ix->filt.reserve(ix->h_fl_off[L]));
    CU_TRY(cudaMemcpyAsync(ix->fl_off.p, ix->h_fl_off.data(), 8 * (L + 1), cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(ix->fl_mask.p, flm.data(), 4 * L, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemsetAsync(ix->filt.p, 0, 4 * ix->h_fl_off[L], st));
    CU_TRY(launch_hash_build(ix->boff.p, ix->ukeys.p, L, ix->M, ix->KW, maxB, ix->foff.p, ix->fbits.p, ix->rmul.p,
                             ix->hoff.p, ix->hmask.p, ix->hslots.p, ix->filt.p, ix->fl_off.p, ix->fl_mask.p,
                             ix->err.p, st));
    return CULSH_OK;
}

inline uint16_t bf16_bits_rn(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    const uint32_t bias = 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)((u + bias) >> 16);
}
inline float bf16_to_float(uint16_t h) {
    const uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// Index projection on the tensor cores when the shape allows it. On success
// ws_codes holds every code and cmin/cmax their ranges, exactly as the SIMT
// kernel would produce; *done stays false when the caller must run the SIMT
// kernel instead (shape not covered, CULSH_PROJECT_SIMT set, non-finite data,
// a device wait gave up or the recomputation list overflowed).
int project_tensor_cores(culsh_index* ix, const float* dX, cudaStream_t st, bool* done) {
    *done = false;
    ix->tc_recomputed = -1;
    if (getenv("CULSH_PROJECT_SIMT")) return CULSH_OK;
    const int N = ix->N, D = ix->D, LM = ix->L * ix->M;
    int dev = 0, sms = 0, maxsm = 0, major = 0;
    CU_TRY(cudaGetDevice(&dev));
    CU_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CU_TRY(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    CU_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    if (major < 10) return CULSH_OK;
    // Resident form when the bf16 projection matrix fits shared memory,
    // streaming form (K slices of X and A, column blocks) otherwise.
    const TcPlan rp = tc_plan(N, D, LM, sms, maxsm);
    const TcStreamPlan sp = rp.ok ? TcStreamPlan{} : tc_plan_stream(N, D, LM, sms, maxsm);
    if (!rp.ok && !sp.ok) return CULSH_OK;
    const bool stream = !rp.ok;
    struct {
        int Dp, LMp, grid;
    } p = {stream ? sp.Dp : rp.Dp, stream ? sp.LMp : rp.LMp, stream ? sp.grid : rp.grid};
    // Host split of the projection matrix and upper bounds of its column norms.
    std::vector<uint16_t> ah((size_t)p.LMp * p.Dp, 0), al((size_t)p.LMp * p.Dp, 0);
    std::vector<float> an(LM);
    for (int c = 0; c < LM; ++c) {
        double ss = 0.0;
        for (int d = 0; d < D; ++d) {
            const float v = ix->A[(size_t)c * D + d];
            const uint16_t h = bf16_bits_rn(v);
            ah[(size_t)c * p.Dp + d] = h;
            al[(size_t)c * p.Dp + d] = bf16_bits_rn(v - bf16_to_float(h));
            ss += (double)v * v;
        }
        an[c] = std::nextafter((float)(std::sqrt(ss) * (1.0 + 1e-6)), INFINITY);
    }
    CU_TRY(ix->ws_ah.reserve(ah.size()));
    CU_TRY(ix->ws_al.reserve(al.size()));
    CU_TRY(ix->ws_anorm.reserve(LM));
    CU_TRY(cudaMemcpyAsync(ix->ws_ah.p, ah.data(), 2 * ah.size(), cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(ix->ws_al.p, al.data(), 2 * al.size(), cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(ix->ws_anorm.p, an.data(), 4 * LM, cudaMemcpyHostToDevice, st));
    const size_t nx = (size_t)N * p.Dp;
    CU_TRY(ix->ws_xh.reserve(nx));
    CU_TRY(ix->ws_xl.reserve(nx));
    CU_TRY(ix->ws_xnorm.reserve(N));
    CU_TRY(ix->ws_tcflags.reserve(4));
    CU_TRY(cudaMemsetAsync(ix->ws_tcflags.p, 0, 16, st));
    CU_TRY(launch_split_rows(dX, N, D, p.Dp, ix->ws_xh.p, ix->ws_xl.p, ix->ws_xnorm.p, ix->ws_tcflags.p, st));
    int flags = 0;
    CU_TRY(cudaMemcpyAsync(&flags, ix->ws_tcflags.p, 4, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    if (flags & 2) return CULSH_OK;   // non-finite data: the SIMT kernel reports it
    const int need_lo = flags & 1;
    // Bound on |tensor-core sum - canonical FP32 chain| per unit of sum|x||a|
    // (bounded by |x|_2 |a|_2): split residue, one rounding per summed
    // product, the canonical chain's rounding; 1.25 margin.
    const double u24 = std::ldexp(1.0, -24), u23 = std::ldexp(1.0, -23), u16 = std::ldexp(1.0, -16);
    const double split = need_lo ? 3.02 * u16 : 1.01 * u16;
    const double accum = ((need_lo ? 3.0 : 2.0) * D + 16) * u23;
    const float kappa = (float)(1.25 * ((D + 2) * u24 + split + accum));
    {
        // Predicted share of codes the bound leaves open: a code is open when
        // an integer lies within E / W of its value, E = kappa |x| |a|. Above
        // 6 % the FP32 recomputation costs more than the SIMT projection
        // itself (e.g. D = 960, W = 0.25: 14 %), so the SIMT kernel runs.
        const int ns = (int)std::min<int64_t>(N, 4096);
        std::vector<float> xs(ns);
        CU_TRY(cudaMemcpyAsync(xs.data(), ix->ws_xnorm.p, 4 * (size_t)ns, cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaStreamSynchronize(st));
        std::vector<float> as(an.begin(), an.end());
        std::nth_element(xs.begin(), xs.begin() + ns / 2, xs.end());
        std::nth_element(as.begin(), as.begin() + LM / 2, as.end());
        const double open = 2.0 * (double)kappa * xs[ns / 2] * as[LM / 2] / (double)ix->W;
        ix->tc_predicted_open = open;
        if (open > 0.06 && !getenv("CULSH_PROJECT_TC")) return CULSH_OK;
    }
    // One recomputation region per CTA, sized for 1/6 of its codes.
    const unsigned long long cap = ((unsigned long long)N * LM / 6) / p.grid + 4096;
    CU_TRY(ix->ws_relist.reserve(cap * p.grid));
    CU_TRY(ix->ws_relist_cnt.reserve(p.grid));
    CU_TRY(ix->ws_pmin.reserve((size_t)p.grid * LM));
    CU_TRY(ix->ws_pmax.reserve((size_t)p.grid * LM));
    if (stream)
        CU_TRY(launch_project_tc_stream(sp, need_lo, N, D, LM, ix->ws_xh.p, ix->ws_xl.p, ix->ws_ah.p, ix->ws_al.p,
                                        ix->db.p, ix->ws_anorm.p, ix->ws_xnorm.p, ix->W, kappa, ix->ws_codes.p,
                                        ix->ws_pmin.p, ix->ws_pmax.p, ix->ws_relist.p, cap, ix->ws_relist_cnt.p,
                                        ix->err.p, st));
    else
        CU_TRY(launch_project_tc(rp, need_lo, N, D, LM, ix->ws_xh.p, ix->ws_xl.p, ix->ws_ah.p, ix->ws_al.p, ix->db.p,
                                 ix->ws_anorm.p, ix->ws_xnorm.p, ix->W, kappa, ix->ws_codes.p, ix->ws_pmin.p,
                                 ix->ws_pmax.p, ix->ws_relist.p, cap, ix->ws_relist_cnt.p, ix->err.p, st));
    CU_TRY(launch_minmax_reduce(ix->ws_pmin.p, ix->ws_pmax.p, p.grid, LM, ix->cmin.p, ix->cmax.p, st));
    std::vector<unsigned int> cnt(p.grid);
    int err = 0;
    CU_TRY(cudaMemcpyAsync(cnt.data(), ix->ws_relist_cnt.p, 4 * p.grid, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaMemcpyAsync(&err, ix->err.p, 4, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    unsigned long long nre = 0;
    bool overflow = false;
    for (unsigned int c : cnt) {
        nre += c;
        overflow |= c > cap;
    }
    if (err != 0 || overflow) {
        CU_TRY(cudaMemsetAsync(ix->err.p, 0, sizeof(int), st));
        return CULSH_OK;   // fall back to the SIMT kernel
    }
    if (nre)
        CU_TRY(launch_tc_recompute(dX, N, D, LM, ix->dA.p, ix->db.p, ix->W, ix->ws_relist.p, cap, ix->ws_relist_cnt.p,
                                   p.grid, ix->ws_codes.p, ix->cmin.p, ix->cmax.p, ix->err.p, st));
    ix->tc_recomputed = (long long)nre;
    ix->tc_need_lo = need_lo;
    *done = true;
    return CULSH_OK;
}

// Orders every table's points by packed key (ties by id), the order of the
// reference's LSD row sort (cuLSH_Indexing.cu:71-93). Multi-word keys first
// take the digit passes over the top word alone (moving 8 bytes per point a
// pass instead of 4 (KW + 1)), gather the lower words into sorted order, and
// order each run of equal top words by (lower words, id); a run longer than
// run_max_len() or more runs than the lists hold sends the build through the
// passes over every word instead. On return *skeys holds the sorted keys
// ([KW][L*N]) and ix->ids the sorted ids.
int sort_keys(culsh_index* ix, int N, int passes, cudaStream_t st, const uint32_t** skeys) {
    const int L = ix->L, KW = ix->KW;
    const size_t LN = (size_t)L * N;
    SortBuffers sb;
    sb.keys[0] = ix->ws_keys[0].p;
    sb.keys[1] = ix->ws_keys[1].p;
    sb.vals[0] = ix->ids.p;
    sb.vals[1] = ix->ws_vals.p;
    sb.hist = ix->ws_hist.p;
    sb.base = ix->ws_base.p;
    sb.status = ix->ws_status.p;
    sb.err = ix->err.p;
    sb.h_hist = ix->h_sort_hist.p;
    sb.h_hist_words = ix->h_sort_hist.n;
    const int top_passes = passes - 4 * (KW - 1);
    ix->sort_form = 0;
    if (KW >= 2 && top_passes >= 1 && !getenv("CULSH_SORT_ALL_WORDS")) {
        SortBuffers sa = sb;
        sa.keys[0] = ix->ws_keys[0].p + (KW - 1) * LN;   // read first, then a ping-pong slot
        sa.keys[1] = ix->ws_keys[1].p + (KW - 1) * LN;
        bool alt = false;
        CU_TRY(run_segmented_sort(sa, N, L, 1, top_passes, &alt, st));
        const uint32_t* top = alt ? sa.keys[1] : sa.keys[0];
        if (alt) ix->ids.swap(ix->ws_vals);
        // ws_keys[0]'s lower words are still in point order; its top slot may
        // hold sorted top words (read before being overwritten: other buffer)
        CU_TRY(launch_gather_lower(ix->ws_keys[0].p, ix->ids.p, top, N, L, KW, ix->ws_keys[1].p, st));
        const unsigned int tcap = (unsigned int)std::min<size_t>(LN / 2 + 1, (size_t)1 << 23);
        const unsigned int scap = (unsigned int)std::min<size_t>(LN / 9 + 1, (size_t)1 << 21);
        const unsigned int lcap = (unsigned int)std::min<size_t>(LN / 33 + 1, (size_t)1 << 18);
        const size_t rcap = (size_t)tcap + scap + lcap;
        CU_TRY(ix->ws_run_pos.reserve(rcap));
        CU_TRY(ix->ws_run_len.reserve(rcap));
        CU_TRY(ix->ws_run_cnt.reserve(4));
        CU_TRY(ix->h_run_cnt.reserve(4));
        RunLists rl;
        rl.tpos = ix->ws_run_pos.p;
        rl.tlen = ix->ws_run_len.p;
        rl.tcap = tcap;
        rl.spos = ix->ws_run_pos.p + tcap;
        rl.slen = ix->ws_run_len.p + tcap;
        rl.scap = scap;
        rl.lpos = ix->ws_run_pos.p + tcap + scap;
        rl.llen = ix->ws_run_len.p + tcap + scap;
        rl.lcap = lcap;
        rl.cnt = ix->ws_run_cnt.p;
        const uint32_t* stop = ix->ws_keys[1].p + (KW - 1) * LN;
        CU_TRY(launch_run_find(stop, N, L, rl, st));
        CU_TRY(cudaMemcpyAsync(ix->h_run_cnt.p, rl.cnt, 4 * sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaStreamSynchronize(st));
        const unsigned int* hc = ix->h_run_cnt.p;
        if (hc[3] == 0) {
            CU_TRY(launch_run_sorts(rl, hc, N, L, KW, ix->ws_keys[1].p, ix->ids.p, st));
            ix->sort_form = 1;
            *skeys = ix->ws_keys[1].p;
            return CULSH_OK;
        }
        // a run too long to order in shared memory: repack, sort every word
        CU_TRY(launch_pack_keys(ix->ws_codes.p, N, L, ix->M, KW, ix->cmin.p, ix->fbits.p, ix->foff.p,
                                ix->ws_keys[0].p, ix->ids.p, st));
        sb.vals[0] = ix->ids.p;
        sb.vals[1] = ix->ws_vals.p;
        ix->sort_form = 2;
    }
    bool alt = false;
    CU_TRY(run_segmented_sort(sb, N, L, KW, passes, &alt, st));
    *skeys = ix->ws_keys[alt ? 1 : 0].p;
    if (alt) ix->ids.swap(ix->ws_vals);
    return CULSH_OK;
}

// Index build from a device-resident dataset (cuLSH_HashTables.cu:486-520).
int build_device(culsh_index* ix, const float* dX, cudaStream_t st, FILE* dbg) {
    const int N = ix->N, D = ix->D, L = ix->L, M = ix->M, LM = L * M;
    const double t0 = seconds_now();
    ix->big_valid = false;
    for (auto& e : ix->bev)
        if (!e) CU_TRY(cudaEventCreate(&e));
    CU_TRY(cudaEventRecord(ix->bev[0], st));
    TRY(upload_projection(ix, st));
    CU_TRY(ix->err.reserve(1));
    CU_TRY(cudaMemsetAsync(ix->err.p, 0, sizeof(int), st));
    CU_TRY(ix->ws_codes.reserve((size_t)LM * N));
    CU_TRY(ix->cmin.reserve(LM));
    CU_TRY(ix->cmax.reserve(LM));
    bool tc_done = false;
    TRY(project_tensor_cores(ix, dX, st, &tc_done));
    if (!tc_done) {
        const int gx = project_grid_x(N);
        CU_TRY(ix->ws_pmin.reserve((size_t)gx * LM));
        CU_TRY(ix->ws_pmax.reserve((size_t)gx * LM));
        CU_TRY(launch_project_fp32(dX, N, D, ix->dAT.p, ix->lmp, ix->db.p, LM, ix->W, ix->ws_codes.p, nullptr,
                                   ix->ws_pmin.p, ix->ws_pmax.p, ix->err.p, st));
        CU_TRY(launch_minmax_reduce(ix->ws_pmin.p, ix->ws_pmax.p, gx, LM, ix->cmin.p, ix->cmax.p, st));
    }
    ix->h_cmin.resize(LM);
    ix->h_cmax.resize(LM);
    CU_TRY(cudaMemcpyAsync(ix->h_cmin.data(), ix->cmin.p, 4 * LM, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaMemcpyAsync(ix->h_cmax.data(), ix->cmax.p, 4 * LM, cudaMemcpyDeviceToHost, st));
    TRY(read_err_flag(ix, st, "index"));
    int passes = 0;
    TRY(compute_layout(ix, &passes));
    TRY(upload_layout(ix, st));
    ix->sort_passes = passes;
    CU_TRY(cudaEventRecord(ix->bev[1], st));
    if (dbg)
        fprintf(dbg, "[HashTables::index]\tprojected %d points onto %d tables x %d columns (%s, %lld codes recomputed); "
                "%d key words, %d sort passes\n",
                N, L, M, ix->tc_recomputed >= 0 ? "tensor cores" : "FP32 SIMT", ix->tc_recomputed, ix->KW, passes);

    // Pack keys and sort all tables at once.
    const size_t LN = (size_t)L * N;
    CU_TRY(ix->ws_keys[0].reserve(LN * ix->KW));
    CU_TRY(ix->ws_keys[1].reserve(LN * ix->KW));
    CU_TRY(ix->ws_vals.reserve(LN));
    CU_TRY(ix->ids.reserve(LN));
    CU_TRY(launch_pack_keys(ix->ws_codes.p, N, L, M, ix->KW, ix->cmin.p, ix->fbits.p, ix->foff.p, ix->ws_keys[0].p,
                            ix->ids.p, st));
    const int hp = std::max(passes, 1);
    CU_TRY(ix->ws_hist.reserve((size_t)L * hp * 256));
    CU_TRY(ix->ws_base.reserve((size_t)L * hp * 256));
    CU_TRY(ix->ws_status.reserve(sort_status_words(N, L)));
    CU_TRY(ix->h_sort_hist.reserve((size_t)L * hp * 256));
    CU_TRY(cudaEventRecord(ix->bev[2], st));
    const uint32_t* skeys = nullptr;
    TRY(sort_keys(ix, N, passes, st, &skeys));
    CU_TRY(cudaEventRecord(ix->bev[3], st));

    // Run-length bucketing.
    const int tiles = (N + 4095) / 4096;
    CU_TRY(ix->ws_tcnt.reserve((size_t)L * tiles));
    CU_TRY(ix->ws_toff.reserve((size_t)L * tiles));
    CU_TRY(ix->ws_nb.reserve(L));
    CU_TRY(launch_rl_count(skeys, N, L, ix->KW, ix->ws_tcnt.p, ix->ws_toff.p, ix->ws_nb.p, st));
    ix->buckets.assign(L, 0);
    CU_TRY(cudaMemcpyAsync(ix->buckets.data(), ix->ws_nb.p, 4 * L, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    ix->h_boff.assign(L + 1, 0);
    int64_t maxB = 0;
    for (int l = 0; l < L; ++l) {
        ix->h_boff[l + 1] = ix->h_boff[l] + ix->buckets[l];
        maxB = std::max<int64_t>(maxB, ix->buckets[l]);
    }
    const uint64_t totB = ix->h_boff[L];
    CU_TRY(ix->boff.reserve(L + 1));
    CU_TRY(cudaMemcpyAsync(ix->boff.p, ix->h_boff.data(), 8 * (L + 1), cudaMemcpyHostToDevice, st));
    CU_TRY(ix->starts.reserve(totB));
    CU_TRY(ix->sizes.reserve(totB));
    CU_TRY(ix->ukeys.reserve(totB * ix->KW));
    CU_TRY(launch_rl_write(skeys, N, L, ix->KW, ix->ws_toff.p, ix->boff.p, ix->starts.p, ix->ukeys.p, st));
    CU_TRY(ix->maxb.reserve(1));
    CU_TRY(cudaMemsetAsync(ix->maxb.p, 0, sizeof(uint32_t), st));
    CU_TRY(launch_bucket_sizes(ix->boff.p, ix->starts.p, N, L, maxB, ix->sizes.p, ix->maxb.p, st));
    CU_TRY(ix->h_maxb.reserve(1));   // pinned: the copy does not block the host mid-build
    CU_TRY(cudaMemcpyAsync(ix->h_maxb.p, ix->maxb.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    TRY(build_hash(ix, st));
    CU_TRY(cudaEventRecord(ix->bev[4], st));
    TRY(read_err_flag(ix, st, "index"));   // synchronises the stream
    ix->max_bucket = *ix->h_maxb.p;
    ix->indexed = ix->dev_valid = true;
    ix->host_valid = false;
    ix->built_once = true;
    if (dbg) {
        for (int l = 0; l < L; ++l)
            fprintf(dbg, "[HashTables::index]\ttable %d/%d -----> %u distinct buckets\n", l + 1, L, ix->buckets[l]);
        fprintf(dbg, "[HashTables::index]\tbuilt in %.3f ms\n", 1e3 * (seconds_now() - t0));
    }
    return CULSH_OK;
}

// Host copies of the bucket arrays (getters, save) from the device index.
int ensure_host(culsh_index* ix) {
    if (ix->host_valid) return CULSH_OK;
    if (!ix->dev_valid) return fail(CULSH_ERR_STATE, "Pointers to bucket objects are null. Have you performed indexing???");
    TRY(ensure_stream(&ix->stream));
    cudaStream_t st = ix->stream;
    const int L = ix->L, N = ix->N, M = ix->M;
    int64_t maxB = 0;
    for (int l = 0; l < L; ++l) maxB = std::max<int64_t>(maxB, ix->buckets[l]);
    CU_TRY(ix->dcodes.reserve(ix->h_boff[L] * M));
    CU_TRY(launch_decode_codes(ix->boff.p, ix->ukeys.p, L, M, ix->KW, maxB, ix->cmin.p, ix->fbits.p, ix->foff.p,
                               ix->dcodes.p, st));
    ix->h_ids.assign(L, {});
    ix->h_starts.assign(L, {});
    ix->h_sizes.assign(L, {});
    ix->h_codes.assign(L, {});
    for (int l = 0; l < L; ++l) {
        const uint64_t B = ix->buckets[l], bo = ix->h_boff[l];
        ix->h_ids[l].resize(N);
        ix->h_starts[l].resize(B);
        ix->h_sizes[l].resize(B);
        ix->h_codes[l].resize(B * M);
        CU_TRY(cudaMemcpyAsync(ix->h_ids[l].data(), ix->ids.p + (size_t)l * N, 4 * (size_t)N, cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaMemcpyAsync(ix->h_starts[l].data(), ix->starts.p + bo, 4 * B, cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaMemcpyAsync(ix->h_sizes[l].data(), ix->sizes.p + bo, 4 * B, cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaMemcpyAsync(ix->h_codes[l].data(), ix->dcodes.p + bo * M, 4 * B * M, cudaMemcpyDeviceToHost, st));
    }
    CU_TRY(cudaStreamSynchronize(st));
    ix->host_valid = true;
    return CULSH_OK;
}

// Device index from host arrays (after load()).
int ensure_device(culsh_index* ix, cudaStream_t st) {
    if (ix->dev_valid) return upload_projection(ix, st);
    if (!ix->host_valid) return fail(CULSH_ERR_STATE, "No index: have you performed indexing or loaded a file???");
    const int L = ix->L, N = ix->N, M = ix->M, LM = L * M;
    ix->big_valid = false;
    TRY(upload_projection(ix, st));
    CU_TRY(ix->err.reserve(1));
    CU_TRY(cudaMemsetAsync(ix->err.p, 0, sizeof(int), st));
    ix->h_boff.assign(L + 1, 0);
    int64_t maxB = 0;
    ix->max_bucket = 0;
    for (int l = 0; l < L; ++l) {
        ix->h_boff[l + 1] = ix->h_boff[l] + ix->buckets[l];
        maxB = std::max<int64_t>(maxB, ix->buckets[l]);
        for (uint32_t v : ix->h_sizes[l]) ix->max_bucket = std::max(ix->max_bucket, v);
    }
    const uint64_t totB = ix->h_boff[L];
    CU_TRY(ix->ids.reserve((size_t)L * N));
    CU_TRY(ix->boff.reserve(L + 1));
    CU_TRY(ix->starts.reserve(totB));
    CU_TRY(ix->sizes.reserve(totB));
    CU_TRY(ix->dcodes.reserve(totB * M));
    CU_TRY(cudaMemcpyAsync(ix->boff.p, ix->h_boff.data(), 8 * (L + 1), cudaMemcpyHostToDevice, st));
    for (int l = 0; l < L; ++l) {
        const uint64_t B = ix->buckets[l], bo = ix->h_boff[l];
        CU_TRY(cudaMemcpyAsync(ix->ids.p + (size_t)l * N, ix->h_ids[l].data(), 4 * (size_t)N, cudaMemcpyHostToDevice, st));
        CU_TRY(cudaMemcpyAsync(ix->starts.p + bo, ix->h_starts[l].data(), 4 * B, cudaMemcpyHostToDevice, st));
        CU_TRY(cudaMemcpyAsync(ix->sizes.p + bo, ix->h_sizes[l].data(), 4 * B, cudaMemcpyHostToDevice, st));
        CU_TRY(cudaMemcpyAsync(ix->dcodes.p + bo * M, ix->h_codes[l].data(), 4 * B * M, cudaMemcpyHostToDevice, st));
    }
    ix->h_cmin.assign(LM, INT_MAX);
    ix->h_cmax.assign(LM, INT_MIN);
    CU_TRY(ix->cmin.reserve(LM));
    CU_TRY(ix->cmax.reserve(LM));
    CU_TRY(cudaMemcpyAsync(ix->cmin.p, ix->h_cmin.data(), 4 * LM, cudaMemcpyHostToDevice, st));
    CU_TRY(cudaMemcpyAsync(ix->cmax.p, ix->h_cmax.data(), 4 * LM, cudaMemcpyHostToDevice, st));
    CU_TRY(launch_codes_minmax(ix->boff.p, ix->dcodes.p, L, M, maxB, ix->cmin.p, ix->cmax.p, ix->err.p, st));
    CU_TRY(cudaMemcpyAsync(ix->h_cmin.data(), ix->cmin.p, 4 * LM, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaMemcpyAsync(ix->h_cmax.data(), ix->cmax.p, 4 * LM, cudaMemcpyDeviceToHost, st));
    TRY(read_err_flag(ix, st, "load"));
    int passes = 0;
    TRY(compute_layout(ix, &passes));
    TRY(upload_layout(ix, st));
    CU_TRY(ix->ukeys.reserve(totB * ix->KW));
    CU_TRY(launch_pack_from_codes(ix->boff.p, ix->dcodes.p, L, M, ix->KW, maxB, ix->cmin.p, ix->fbits.p, ix->foff.p,
                                  ix->ukeys.p, st));
    TRY(build_hash(ix, st));
    TRY(read_err_flag(ix, st, "load"));
    ix->dev_valid = true;
    return CULSH_OK;
}

// Whether every code range of the index sits below 2^24 in magnitude (the
// fast probe kernel's integer +-1 then equals the reference's float +-1).
int small_codes(const culsh_index* ix) {
    for (size_t i = 0; i < ix->h_cmin.size(); ++i)
        if (ix->h_cmin[i] <= -(1 << 24) + 2 || ix->h_cmax[i] >= (1 << 24) - 2) return 0;
    return 1;
}

LookupView lookup_view(const culsh_index* ix) {
    LookupView lv;
    lv.L = ix->L;
    lv.M = ix->M;
    lv.KW = ix->KW;
    lv.cmin = ix->cmin.p;
    lv.cmax = ix->cmax.p;
    lv.fbits = ix->fbits.p;
    lv.foff = ix->foff.p;
    lv.boff = ix->boff.p;
    lv.starts = ix->starts.p;
    lv.sizes = ix->sizes.p;
    lv.ukeys = ix->ukeys.p;
    lv.hslots = ix->hslots.p;
    lv.hoff = ix->hoff.p;
    lv.hmask = ix->hmask.p;
    lv.filt = ix->filt.p;
    lv.fl_off = ix->fl_off.p;
    lv.fl_mask = ix->fl_mask.p;
    lv.funit = ix->funit.p;
    lv.rmul = ix->rmul.p;
    return lv;
}

constexpr size_t kArenaInitialWords = size_t(1) << 24;   // 64 MB of overflow hash sets

// Upper bound on the overflow arena, in 32-bit words. CULSH_ARENA_WORDS lowers
// it (admission tests force the deferral and out-of-memory paths with it).
size_t arena_cap_words() {
    const char* e = getenv("CULSH_ARENA_WORDS");
    if (e) {
        const long long v = atoll(e);
        if (v > 0) return (size_t)v;
    }
    return ~size_t(0);
}

}  // namespace

std::mutex& culsh::alloc_capture_mutex() {
    static std::mutex mu;
    return mu;
}

int culsh::set_last_error(int code, const char* msg) { return fail(code, "%s", msg); }

namespace {

// CULSH_CANDIDATES_PER_QUERY forces the per-query candidate kernel (one
// block per query; the tests run both forms).
int forced_per_query() { return getenv("CULSH_CANDIDATES_PER_QUERY") != nullptr; }

constexpr int kWsPartitions = 64;              // most partitions of one query

// Statistics words of a search (device, cleared by its first kernel, copied
// to the host after it): [0] unique and [1] non-unique candidate totals,
// [2] overflow-arena top, [3] deferred queries, [4] work-stealing item
// counter (low) and overflow flag (high), [5] items, [6] BF16 re-checks,
// [7] dense queries (low) and their claim counter (high), [8..9] the dense
// queries' k-NN row state, [10] tensor-core fallback queries, [11] its error
// flags, [12..13] totals of re-runs that must not count twice.
constexpr int kStatWords = 16;
constexpr size_t kWsPartialBytes = size_t(64) << 20;

// CULSH_WS_PARTITIONS (1..64) and CULSH_WS_ITEMS lower the partition count
// and the item capacity; the tests use them to reach both overflow re-runs.
int env_int(const char* name, int lo, int hi, int dflt) {
    const char* e = getenv(name);
    if (!e) return dflt;
    const long long v = atoll(e);
    return v < lo ? lo : (v > hi ? hi : (int)v);
}

// Everything the enqueued search work depends on: kernel arguments, launch
// shapes, buffers, events. Built zero-filled and compared bytewise, it is
// the key of the cached CUDA graph.
struct SearchPlan {
    const float* dQ;
    int Q, D, LM, proj_tile, lmp;
    float W;
    float* xcopy;   // fused host-copy form: dQ is the caller's host rows, copied here on the way
    const float* AT;
    const float* b;
    float* vals;
    ProbeArgs pa;
    int probe_generic;
    int use_ws, ws_grid, use_dense, dense_grid;
    int use_knn;        // dense queries on the tensor cores (membership rows + masked GEMM)
    uint32_t* kbm;      // their membership rows
    KnnSearch kn;
    CandArgs ca;
    WsArgs wa;
    unsigned long long* stats;
    unsigned long long* h_stats;
    unsigned long long* cnu;
    cudaEvent_t ev[5];  // stage boundaries; ev[4]: membership rows done (tensor-core path)
    int stage_events;   // 0: no stage events in the graph (they cost a few microseconds each)
};

static_assert(sizeof(SearchPlan) <= kPlanBytes, "graph key buffer too small");

// Dataset rows of the tensor-core k-NN path (bf16 parts, weights, flags),
// made once per dataset. The stream is drained before they are published:
// searches on other streams read them as soon as they see them.
int ensure_knn_rows(culsh_index* ix, cudaStream_t st) {
    if (ix->kx_valid) return CULSH_OK;
    const int N = ix->N, D = ix->D, Dp = (D + 63) / 64 * 64;
    const int64_t pad = ((int64_t)N + 255) / 256 * 256;
    CU_TRY(ix->kx_h.reserve((size_t)N * Dp));
    CU_TRY(ix->kx_l.reserve((size_t)N * Dp));
    CU_TRY(ix->kw_exact.reserve((size_t)pad));
    CU_TRY(ix->kw_bound.reserve((size_t)pad));
    CU_TRY(ix->kstate.reserve(1));
    CU_TRY(cudaMemsetAsync(ix->kstate.p, 0, sizeof(KnnState), st));
    CU_TRY(launch_knn_rows_dataset(ix->dev_x(), N, D, Dp, ix->kx_h.p, ix->kx_l.p, ix->kw_exact.p, ix->kw_bound.p, pad,
                                   knn_bound_factor(D), ix->kstate.p, st));
    CU_TRY(cudaMemcpyAsync(&ix->h_kstate, ix->kstate.p, sizeof(KnnState), cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    ix->kx_valid = true;
    return CULSH_OK;
}

// Bucket rows: every bucket of at least big_min ids gets an N-bit row (nwp
// words), which the membership kernel ORs into a dense query's row instead of
// setting the bucket's bits id by id. big_min = max(1024, N/64), where a row
// (N/8 bytes) is at most twice the bucket's ids (4 bytes each); there are then
// at most 64 L rows. CULSH_BIG_ROWS_MIN overrides big_min (0: no rows). Rows
// beyond kBigRowsBytes keep only the largest buckets. Made once per index; the
// stream is drained before they are published.
constexpr size_t kBigRowsBytes = size_t(1) << 30;

int ensure_big_rows(culsh_index* ix, int nwp, cudaStream_t st) {
    if (ix->big_valid) return CULSH_OK;
    const int L = ix->L, N = ix->N;
    ix->nbig = 0;
    ix->big_min = UINT32_MAX;
    long long bmin = std::max(1024ll, (long long)N / 64);
    if (const char* e = getenv("CULSH_BIG_ROWS_MIN")) bmin = atoll(e);
    if (bmin <= 0 || (long long)ix->max_bucket < bmin) {
        ix->big_valid = true;
        return CULSH_OK;
    }
    const uint64_t totB = ix->h_boff[L];
    const unsigned int cap = (unsigned int)std::min<long long>((long long)L * (N / bmin) + 1, 1ll << 20);
    CU_TRY(ix->big_gi.reserve(cap));
    CU_TRY(ix->big_sz.reserve(cap));
    CU_TRY(ix->big_cnt.reserve(1));
    CU_TRY(cudaMemsetAsync(ix->big_cnt.p, 0, sizeof(unsigned int), st));
    CU_TRY(launch_big_find(ix->sizes.p, totB, (uint32_t)bmin, ix->big_gi.p, ix->big_sz.p, ix->big_cnt.p, cap, st));
    unsigned int cnt = 0;
    CU_TRY(cudaMemcpyAsync(&cnt, ix->big_cnt.p, sizeof(cnt), cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    cnt = std::min(cnt, cap);
    std::vector<uint64_t> gi(cnt);
    std::vector<uint32_t> sz(cnt);
    CU_TRY(cudaMemcpyAsync(gi.data(), ix->big_gi.p, 8 * (size_t)cnt, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaMemcpyAsync(sz.data(), ix->big_sz.p, 4 * (size_t)cnt, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    std::vector<uint32_t> ord(cnt);
    for (uint32_t i = 0; i < cnt; ++i) ord[i] = i;
    const size_t row_bytes = 4 * (size_t)nwp;
    const size_t keep = std::min<size_t>({(size_t)cnt, kBigRowsBytes / row_bytes, 65535});
    uint32_t kept_min = (uint32_t)bmin;
    if (keep < cnt) {
        // the largest buckets; a bucket of the smallest kept size without a
        // row is still served id by id
        std::sort(ord.begin(), ord.end(), [&](uint32_t x, uint32_t y) { return sz[x] > sz[y]; });
        ord.resize(keep);
        kept_min = keep ? sz[ord.back()] : UINT32_MAX;
    }
    std::sort(ord.begin(), ord.end(), [&](uint32_t x, uint32_t y) { return gi[x] < gi[y]; });
    std::vector<uint64_t> hg(keep);
    std::vector<int32_t> ht(keep);
    for (size_t r = 0; r < keep; ++r) {
        hg[r] = gi[ord[r]];
        ht[r] = (int32_t)(std::upper_bound(ix->h_boff.begin(), ix->h_boff.begin() + L + 1, hg[r]) -
                          ix->h_boff.begin()) - 1;
    }
    if (keep > 0) {
        CU_TRY(ix->big_tl.reserve(keep));
        CU_TRY(ix->big_rows.reserve(keep * (size_t)nwp));
        CU_TRY(cudaMemcpyAsync(ix->big_gi.p, hg.data(), 8 * keep, cudaMemcpyHostToDevice, st));
        CU_TRY(cudaMemcpyAsync(ix->big_tl.p, ht.data(), 4 * keep, cudaMemcpyHostToDevice, st));
        CU_TRY(cudaMemsetAsync(ix->big_rows.p, 0, keep * row_bytes, st));
        CU_TRY(launch_big_fill(ix->big_gi.p, ix->big_tl.p, (int)keep, ix->starts.p, ix->sizes.p, ix->ids.p, N,
                               ix->big_rows.p, nwp, st));
        CU_TRY(cudaStreamSynchronize(st));
    }
    ix->nbig = (int)keep;
    ix->big_min = keep ? kept_min : UINT32_MAX;
    ix->big_valid = true;
    return CULSH_OK;
}

// Whether the dataset's values allow the exact form (integers of magnitude
// <= 256, D max|v|^2 < 2^24 and D (max - min)^2 < 2^24); the queries must
// qualify too, which the kernels check on the device.
bool knn_dataset_exact(const culsh_index* ix) {
    const KnnState& k = ix->h_kstate;
    if (k.flags & (kKnnNotSmallInt | kKnnNonFinite) || k.mneg == 0 || k.mpos == 0) return false;
    const long long lo = 257 - k.mneg, hi = k.mpos - 257, mag = std::max(-lo, hi);
    return (long long)ix->D * mag * mag < (1ll << 24) && (long long)ix->D * (hi - lo) * (hi - lo) < (1ll << 24);
}

// Membership rows above this size send the dense queries to the SIMT kernel.
constexpr size_t kKnnMaxBitmapBytes = size_t(16) << 30;

// Plans the tensor-core path for the dense queries of a search of Q queries
// (sets *ok); it declines dimensions above 128, K above kMaxKnnK, datasets
// whose N-bit bitmap does not fit a block's shared memory and membership rows
// above kKnnMaxBitmapBytes.
int plan_knn(culsh_search* s, SearchPlan& P, int Q, int32_t* d_ids, float* d_d, cudaStream_t st, bool* ok) {
    *ok = false;
    culsh_index* ix = s->ix;
    KnnSearch& k = P.kn;
    k.N = ix->N;
    k.D = ix->D;
    k.K = s->K;
    k.Qcap = (Q + 2 * kKnnTileQ - 1) / (2 * kKnnTileQ) * (2 * kKnnTileQ);   // whole 256-query tiles
    k.grid = s->sms;
    if (!knn_plan(k, s->smem_optin)) return CULSH_OK;
    if (bitmap_smem_bytes(ix->N) + 8192 > (size_t)s->smem_optin) return CULSH_OK;
    const size_t bm_words = (size_t)k.Qcap * k.nwp;
    if (4 * bm_words > kKnnMaxBitmapBytes) return CULSH_OK;
    TRY(ensure_knn_rows(ix, st));
    if (ix->h_kstate.flags & kKnnNonFinite) return CULSH_OK;
    TRY(ensure_big_rows(ix, k.nwp, st));
    k.exact_possible = knn_dataset_exact(ix) && k.ops_exact > 0;
    k.C = knn_bound_factor(ix->D);
    CU_TRY(s->kbm.reserve(bm_words));
    CU_TRY(s->kq_h.reserve((size_t)k.Qcap * k.Dp));
    CU_TRY(s->kq_l.reserve((size_t)k.Qcap * k.Dp));
    CU_TRY(s->kq_sq.reserve(k.Qcap));
    CU_TRY(s->kq_base.reserve(k.Qcap));
    CU_TRY(s->kq_bound.reserve(k.Qcap));
    CU_TRY(s->kpart_key.reserve(knn_part_entries(k)));
    CU_TRY(s->kpart_id.reserve(knn_part_entries(k)));
    CU_TRY(s->kpart_n.reserve(knn_part_lists(k)));
    CU_TRY(s->kfallback.reserve(k.Qcap));
    k.xh = ix->kx_h.p;
    k.xl = ix->kx_l.p;
    k.w_exact = ix->kw_exact.p;
    k.w_bound = ix->kw_bound.p;
    k.dstate = ix->kstate.p;
    k.X = ix->dev_x();
    k.queries = P.ca.queries;
    k.dense_q = s->dense_q.p;
    k.n_dense = P.wa.n_dense;
    k.qh = s->kq_h.p;
    k.ql = s->kq_l.p;
    k.qsq = s->kq_sq.p;
    k.qbase = s->kq_base.p;
    k.qbound = s->kq_bound.p;
    k.qstate = reinterpret_cast<KnnState*>(s->stats.p + 8);
    k.bm = s->kbm.p;
    k.part_key = s->kpart_key.p;
    k.part_id = s->kpart_id.p;
    k.part_n = s->kpart_n.p;
    k.out_ids = d_ids;
    k.out_d = d_d;
    k.fallback = s->kfallback.p;
    k.n_fallback = reinterpret_cast<unsigned int*>(s->stats.p + 10);
    k.err = reinterpret_cast<int*>(s->stats.p + 11);
    P.kbm = s->kbm.p;
    *ok = true;
    return CULSH_OK;
}

// Sizes every buffer of a search of Q queries and fills the plan. Allocates
// (when buffers grow) but launches nothing.
int plan_search(culsh_search* s, const float* dQ, int Q, int32_t* d_ids, float* d_d, cudaStream_t st,
                SearchPlan* out, const float* proj_src = nullptr) {
    culsh_index* ix = s->ix;
    const int L = ix->L, M = ix->M, D = ix->D, K = s->K, T = s->T, LM = L * M;
    const float* dX = ix->dev_x();
    if (!dX) return fail(CULSH_ERR_STATE, "the dataset is not on the device");
    for (auto& e : s->ev)
        if (!e) CU_TRY(cudaEventCreate(&e));
    CU_TRY(s->vals.reserve((size_t)LM * Q));
    CU_TRY(s->qb.reserve((size_t)L * Q * T));
    CU_TRY(s->cnu.reserve(Q));
    CU_TRY(s->cu.reserve(Q));
    CU_TRY(s->stats.reserve(kStatWords));
    CU_TRY(s->deferred.reserve(2 * (size_t)Q));
    CU_TRY(s->h_stats.reserve(kStatWords));
    const size_t cap_words = arena_cap_words();
    const size_t init_words = std::min(kArenaInitialWords, cap_words);
    if (s->arena.n < init_words || s->arena.n > cap_words) {
        s->arena.release();
        CU_TRY(s->arena.reserve(init_words));
    }
    const SearchTune& tu = s->tune;
    SearchPlan& P = *out;
    std::memset(&P, 0, sizeof(P));
    P.dQ = dQ;
    P.Q = Q;
    P.D = D;
    P.LM = LM;
    P.proj_tile = tu.proj_tile;
    if (proj_src) {
        // The projection reads the caller's rows (host memory the device can
        // access) and writes them to dQ, which the candidate stage reads.
        P.dQ = proj_src;
        P.xcopy = const_cast<float*>(dQ);
        P.proj_tile = 5;
    }
    P.W = ix->W;
    P.AT = ix->dAT.p;
    P.lmp = ix->lmp;
    P.b = ix->db.p;
    P.vals = s->vals.p;
    P.pa.vals = s->vals.p;
    P.pa.Q = Q;
    P.pa.T = T;
    P.pa.lv = lookup_view(ix);
    P.pa.qbuckets = s->qb.p;
    P.pa.cnu = s->cnu.p;
    P.pa.small_codes = small_codes(ix);
    P.pa.pch = tu.probe_pch;
    P.probe_generic = getenv("CULSH_PROBE_GENERIC") != nullptr;
    {
        // CULSH_PROBE_SPLIT=0/1 overrides the tuning (the tests run both).
        const char* e = getenv("CULSH_PROBE_SPLIT");
        const int form = M <= 16 ? std::min(2, std::max(0, e ? atoi(e) : tu.probe_split)) : 0;
        if (form > 0) {
            CU_TRY(s->ph.reserve((size_t)L * Q * T));
            CU_TRY(s->pmask.reserve((size_t)L * Q * T));
            P.pa.split = form;
            P.pa.ph = s->ph.p;
            P.pa.pmask = s->pmask.p;
            if (form == 1) {
                CU_TRY(s->pctx.reserve(3 * (size_t)L * Q));
                P.pa.pctx = s->pctx.p;
            }
        }
    }
    CandArgs& ca = P.ca;
    ca.X = dX;
    ca.N = ix->N;
    ca.D = D;
    ca.L = L;
    ca.T = T;
    ca.Q = Q;
    ca.K = K;
    ca.queries = dQ;
    ca.qbuckets = s->qb.p;
    ca.boff = ix->boff.p;
    ca.starts = ix->starts.p;
    ca.sizes = ix->sizes.p;
    ca.ids = ix->ids.p;
    ca.cnu = s->cnu.p;
    ca.out_ids = d_ids;
    ca.out_d = d_d;
    ca.cu = s->cu.p;
    ca.totals = s->stats.p;
    ca.arena = s->arena.p;
    ca.arena_words = s->arena.n;
    ca.arena_top = s->stats.p + 2;
    ca.deferred = s->deferred.p;
    ca.n_deferred = reinterpret_cast<unsigned int*>(s->stats.p + 3);
    ca.qlist = nullptr;
    ca.nq = Q;
    P.use_ws = tu.cand_ws && !forced_per_query();
    if (P.use_ws) {
        // A configuration whose item state exceeds the shared memory a block
        // may opt into (large K or D with the wide set) runs per query.
        if (s->smem_optin == 0) {
            int dev = 0;
            CU_TRY(cudaGetDevice(&dev));
            CU_TRY(cudaDeviceGetAttribute(&s->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        }
        const size_t need = ws_smem_bytes(D, K, tu.ws_wt, tu.dist_bf16 ? 1 : 0, tu.ws_slots) + 8192;
        if (need > (size_t)s->smem_optin) P.use_ws = 0;
    }
    if (P.use_ws) {
        // Work-stealing buffers. stats[4] holds the item counter (low word)
        // and the overflow flag (high word), stats[5] the number of items.
        const int pmax = env_int("CULSH_WS_PARTITIONS", 1, kWsPartitions, kWsPartitions);
        const size_t per_item = (size_t)K * 8 + 4 + 4 + 1;
        size_t cap = std::max<size_t>((size_t)Q * 2, kWsPartialBytes / per_item);
        cap = std::min(cap, (size_t)Q * pmax);
        cap = std::min<size_t>(cap, (size_t)env_int("CULSH_WS_ITEMS", 1, 0x7fffffff, 0x7fffffff));
        CU_TRY(s->q_items.reserve(Q));
        CU_TRY(s->q_off.reserve(Q));
        CU_TRY(s->q_done.reserve(Q));
        CU_TRY(s->item_q.reserve(cap));
        CU_TRY(s->item_p.reserve(cap));
        CU_TRY(s->part_n.reserve(cap));
        CU_TRY(s->part_d.reserve(cap * K));
        CU_TRY(s->part_i.reserve(cap * K));
        if (s->sms == 0) {
            int dev = 0;
            CU_TRY(cudaGetDevice(&dev));
            CU_TRY(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev));
        }
        const int bf16 = tu.dist_bf16 ? 1 : 0;
        if (bf16 && !ix->xb_valid) {
            // The bf16 copy and row flags, made once per dataset. The stream
            // is drained before the copy is published: searches on other
            // streams read it as soon as they see it.
            CU_TRY(ix->xb.reserve((size_t)ix->N * D));
            CU_TRY(ix->xflag.reserve((size_t)ix->N));
            CU_TRY(launch_bf16_rows(dX, ix->N, D, ix->xb.p, ix->xflag.p, st));
            CU_TRY(cudaStreamSynchronize(st));
            ix->xb_valid = true;
        }
        // resident CTAs per SM, cached per kernel shape
        const long long okey = ((((long long)D * 4096 + K) * 512 + tu.ws_wt) * 2 + bf16) * 16384 + tu.ws_slots;
        if (s->occ_key != okey) {
            s->occ_val = ws_blocks_per_sm(D, K, tu.ws_wt, bf16, tu.ws_slots);
            s->occ_key = okey;
        }
        const int occ = s->occ_val;
        const int bps = tu.ws_bps > 0 ? std::min(tu.ws_bps, occ) : occ;
        P.ws_grid = s->sms * bps;
        WsArgs& a = P.wa;
        a.X = ca.X;
        a.N = ca.N;
        a.D = D;
        a.L = L;
        a.T = T;
        a.Q = Q;
        a.K = K;
        a.queries = dQ;
        a.qbuckets = ca.qbuckets;
        a.boff = ca.boff;
        a.starts = ca.starts;
        a.sizes = ca.sizes;
        a.ids = ca.ids;
        a.cnu = ca.cnu;
        a.out_ids = d_ids;
        a.out_d = d_d;
        a.cu = ca.cu;
        a.totals = ca.totals;
        a.pmax = pmax;
        a.chunk = (unsigned long long)tu.ws_chunk;
        a.q_items = s->q_items.p;
        a.q_off = s->q_off.p;
        a.q_done = s->q_done.p;
        a.item_q = s->item_q.p;
        a.item_p = s->item_p.p;
        a.part_n = s->part_n.p;
        a.part_d = s->part_d.p;
        a.part_i = s->part_i.p;
        a.item_cap = (unsigned int)cap;
        a.next_item = reinterpret_cast<unsigned int*>(s->stats.p + 4);
        a.overflow = reinterpret_cast<unsigned int*>(s->stats.p + 4) + 1;
        a.n_items = reinterpret_cast<unsigned int*>(s->stats.p + 5);
        a.wt = tu.ws_wt;
        a.slots = tu.ws_slots;
        a.bf16 = bf16;
        // Dense form: queries with at least dense_min non-unique candidates
        // take the tensor-core path (membership rows and a masked GEMM over
        // the whole dataset; default threshold max(4096, N/256)) or, where
        // that path does not apply, the SIMT bitmap kernel (max(32768, N/16)).
        // The tuning or CULSH_DENSE_MIN override the threshold. The dense
        // kernels are launched only when some query could reach it (L*T*largest
        // bucket) and the N-bit bitmap fits the shared memory of a block.
        a.n_dense = reinterpret_cast<unsigned int*>(s->stats.p + 7);
        a.dense_next = reinterpret_cast<unsigned int*>(s->stats.p + 7) + 1;
        const unsigned long long reach = (unsigned long long)L * T * ix->max_bucket;
        auto dense_min_for = [&](bool tc) {
            unsigned long long d = tc ? std::max<unsigned long long>(4096ull, (unsigned long long)ix->N / 256)
                                      : std::max<unsigned long long>(32768ull, (unsigned long long)ix->N / 16);
            if (tu.dense_min > 0) d = (unsigned long long)tu.dense_min;
            if (const char* e = getenv("CULSH_DENSE_MIN")) d = std::max(1ll, atoll(e));
            return d;
        };
        bool knn = false;
        if (tu.dense_tc && !getenv("CULSH_NO_KNN_TC") && reach >= dense_min_for(true)) {
            CU_TRY(s->dense_q.reserve(Q));
            TRY(plan_knn(s, P, Q, d_ids, d_d, st, &knn));
        }
        const unsigned long long dmin = dense_min_for(knn);
        const bool dense_fits = knn || dense_smem_bytes(ix->N, D, K) + 8192 <= (size_t)s->smem_optin;
        P.use_dense = dense_fits && reach >= dmin;
        P.use_knn = P.use_dense && knn;
        a.dense_min = P.use_dense ? dmin : ~0ull;
        if (P.use_dense) {
            CU_TRY(s->dense_q.reserve(Q));
            a.dense_q = s->dense_q.p;
            P.dense_grid = s->sms;
            if (P.use_knn) P.kn.dense_q = s->dense_q.p;
        }
        a.nbig = 0;
        a.big_min = UINT32_MAX;
        if (P.use_knn && ix->nbig > 0 && !getenv("CULSH_NO_BIG_ROWS")) {
            a.big_gi = ix->big_gi.p;
            a.big_rows = ix->big_rows.p;
            a.nbig = ix->nbig;
            a.big_min = ix->big_min;
        }
        if (tu.ws_order) {
            CU_TRY(s->qorder.reserve(Q));
            CU_TRY(s->qorder_bins.reserve(kOrderBins + 1));
            a.order = s->qorder.p;
            a.order_bins = s->qorder_bins.p;
        }
        if (bf16) {
            // |d~ - d| <= c1 d~ + c2 (2 rho b1 + rho^2 b2) with gamma_n = n u / (1 - n u),
            // n = ceil(D/8) + 6 roundings along any path, u = 2^-24:
            // c1 = 2 gamma / (1 - gamma), c2 = (1 + gamma) / (1 - gamma), both
            // rounded up with a 2^-20 margin for the bound's own evaluation.
            const double u = std::ldexp(1.0, -24), nn = (double)((D + 7) / 8 + 6);
            const double g = nn * u / (1.0 - nn * u), margin = 1.0 + std::ldexp(1.0, -20);
            a.xb = ix->xb.p;
            a.xflag = ix->xflag.p;
            a.e_c1 = std::nextafter((float)(2.0 * g / (1.0 - g) * margin), INFINITY);
            a.e_c2 = std::nextafter((float)((1.0 + g) / (1.0 - g) * margin), INFINITY);
            a.rechecked = s->stats.p + 6;
        }
    }
    P.stats = s->stats.p;
    P.h_stats = s->h_stats.p;
    P.cnu = s->cnu.p;
    for (int i = 0; i < 4; ++i) P.ev[i] = s->ev[i];
    P.ev[4] = s->ev[5];
    P.stage_events = s->stage_events ? 1 : 0;
    return CULSH_OK;
}

// Enqueues one search: no allocation, no host synchronisation, so that it
// can be captured into a CUDA graph. Returns the number of kernels launched.
// Inside a capture the stage events become event-record nodes (external
// events); outside one they are ordinary records.
int enqueue_search(const SearchPlan& P, cudaStream_t st, bool capturing, int* launches) {
    const unsigned int evf = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    if (P.stage_events) CU_TRY(cudaEventRecordWithFlags(P.ev[0], st, evf));
    ZeroWords zw;   // the projection kernel clears the non-unique counts and the statistics
    zw.a = P.cnu;
    zw.na = P.Q;
    zw.b = P.stats;
    zw.nb = kStatWords;
    CU_TRY(launch_project_fp32(P.dQ, P.Q, P.D, P.AT, P.lmp, P.b, P.LM, P.W, nullptr, P.vals, nullptr, nullptr,
                               nullptr, st, P.proj_tile, zw, P.xcopy));
    if (P.stage_events) CU_TRY(cudaEventRecordWithFlags(P.ev[1], st, evf));
    CU_TRY(launch_probe(P.pa, st));
    if (P.stage_events) CU_TRY(cudaEventRecordWithFlags(P.ev[2], st, evf));
    if (P.use_ws) {
        if (P.wa.order) CU_TRY(launch_order_queries(P.wa, st));
        CU_TRY(launch_plan_items(P.wa, st));
        CU_TRY(launch_candidates_ws(P.wa, P.ws_grid, st));
        if (P.use_knn) {
            CU_TRY(launch_cand_bitmap(P.wa, P.kbm, P.kn.nwp, P.dense_grid, st));
            if (P.stage_events) CU_TRY(cudaEventRecordWithFlags(P.ev[4], st, evf));
            CU_TRY(launch_knn_search(P.kn, st));
        } else if (P.use_dense) {
            CU_TRY(launch_candidates_dense(P.wa, P.dense_grid, st));
        }
    } else {
        CU_TRY(launch_candidates(P.ca, st));
    }
    if (P.stage_events) CU_TRY(cudaEventRecordWithFlags(P.ev[3], st, evf));
    CU_TRY(cudaMemcpyAsync(P.h_stats, P.stats, 8 * kStatWords, cudaMemcpyDeviceToHost, st));
    const int dense_launches = P.use_knn ? 1 + knn_launches(P.kn) : (P.use_dense ? 1 : 0);
    *launches = (P.use_ws ? 3 + dense_launches + (P.wa.order ? 3 : 0) : 2) + probe_launches(P.pa);
    return CULSH_OK;
}

void drop_graph(culsh_search* s) {
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    if (s->graph) cudaGraphDestroy(s->graph);
    s->gexec = nullptr;
    s->graph = nullptr;
    s->gproj = nullptr;
    s->gsrc = nullptr;
}

// CULSH_NO_GRAPH (or culsh_search_set_graphs(s, 0)) runs the launches
// directly instead of through the cached graph.
bool graphs_enabled(const culsh_search* s, cudaStream_t st) {
    if (!s->use_graphs || st == nullptr || getenv("CULSH_NO_GRAPH")) return false;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return false;
    return true;
}

// The kernel node of g that launches fn, or null.
cudaGraphNode_t find_kernel_node(cudaGraph_t g, const void* fn) {
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return nullptr;
    }
    std::vector<cudaGraphNode_t> nodes(n);
    if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    cudaGraphNode_t found = nullptr;
    for (size_t i = 0; i < n && !found; ++i) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nodes[i], &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams kp;
        if (cudaGraphKernelNodeGetParams(nodes[i], &kp) == cudaSuccess && kp.func == fn) found = nodes[i];
    }
    // a failed query above must not surface as the next launch's error
    cudaGetLastError();
    return found;
}

// Points the instantiated projection node of the fused host-copy form at
// other host rows (later launches of the graph only). False when the node
// cannot be updated: the caller then captures the graph again.
bool set_projection_source(culsh_search* s, const float* src) {
    if (!s->gproj) return false;
    cudaKernelNodeParams kp;
    if (cudaGraphKernelNodeGetParams(s->gproj, &kp) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    void* args[kProjectArgs];
    for (int i = 0; i < kProjectArgs; ++i) args[i] = kp.kernelParams[i];
    const float* x = src;
    args[0] = &x;
    kp.kernelParams = args;
    kp.extra = nullptr;
    if (cudaGraphExecKernelNodeSetParams(s->gexec, s->gproj, &kp) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    s->gsrc = src;
    return true;
}

// Runs the plan: replays the cached graph when the plan is unchanged,
// re-captures it otherwise, or launches directly when graphs are off. In the
// fused host-copy form the caller's rows are not part of the key: a replay
// over other rows updates the projection node in place.
int run_plan(culsh_search* s, const SearchPlan& P, cudaStream_t st) {
    if (!graphs_enabled(s, st)) {
        s->graph_mode = 0;
        return enqueue_search(P, st, false, &s->launches);
    }
    SearchPlan key = P;
    if (P.xcopy) key.dQ = nullptr;
    if (s->gexec && std::memcmp(&key, &s->gplan, sizeof(key)) == 0 &&
        (!P.xcopy || P.dQ == s->gsrc || set_projection_source(s, P.dQ))) {
        CU_TRY(cudaGraphLaunch(s->gexec, st));
        s->launches = s->glaunches;
        s->graph_mode = 2;
        return CULSH_OK;
    }
    drop_graph(s);
    CU_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    int launches = 0;
    const int rc = enqueue_search(P, st, true, &launches);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(st, &g);
    if (rc != CULSH_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (ec != cudaSuccess) return fail(CULSH_ERR_DEVICE, "search graph capture: %s", cudaGetErrorString(ec));
    const cudaError_t ei = cudaGraphInstantiate(&s->gexec, g, 0);
    if (ei != cudaSuccess) {
        cudaGraphDestroy(g);
        s->gexec = nullptr;
        return fail(CULSH_ERR_DEVICE, "search graph instantiation: %s", cudaGetErrorString(ei));
    }
    s->graph = g;
    s->gproj = P.xcopy ? find_kernel_node(g, project_copy_kernel()) : nullptr;
    s->gsrc = P.dQ;
    std::memcpy(&s->gplan, &key, sizeof(key));
    s->glaunches = launches;
    CU_TRY(cudaGraphLaunch(s->gexec, st));
    s->launches = launches;
    s->graph_mode = 1;
    return CULSH_OK;
}

// Runs the per-query candidate kernel over the queries of dl, in chunks whose
// candidate sets fit the overflow arena, growing the arena as far as free
// memory allows (cuLSH_SearchTables.cu:282-306: a query whose candidates
// alone do not fit fails the search). tmpl gives the kernel's arguments; its
// totals pointer decides where the chunk's counts go.
int rerun_queries(culsh_search* s, const CandArgs& tmpl, std::vector<int> dl, int Q, cudaStream_t st) {
    const size_t cap_words = arena_cap_words();
    std::vector<unsigned long long> cnu(Q);
    CU_TRY(cudaMemcpyAsync(cnu.data(), s->cnu.p, 8 * (size_t)Q, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    std::sort(dl.begin(), dl.end());
    size_t need_max = 0, need_all = 0;
    for (int q : dl) {
        need_max = std::max(need_max, cand_arena_words(cnu[q]));
        need_all += cand_arena_words(cnu[q]);
    }
    size_t freeb = 0, totalb = 0;
    CU_TRY(cudaMemGetInfo(&freeb, &totalb));
    size_t avail_words = (freeb + 4 * s->arena.n > (size_t)(64 << 20)) ? (freeb + 4 * s->arena.n - (64 << 20)) / 4 : 0;
    avail_words = std::min(avail_words, cap_words);
    if (need_max > avail_words) {
        for (int q : dl)
            if (cand_arena_words(cnu[q]) == need_max)
                return fail(CULSH_ERR_OUT_OF_MEMORY,
                            "Cannot load all candidates for computation of knn ids of query %d/%d...", q + 1, Q);
    }
    const size_t want = std::min(need_all, avail_words);
    if (want > s->arena.n) {
        std::lock_guard<std::mutex> lk(alloc_capture_mutex());
        s->arena.release();
        CU_TRY(s->arena.reserve(want));
    }
    size_t i = 0;
    while (i < dl.size()) {
        size_t j = i, words = 0;
        while (j < dl.size() && words + cand_arena_words(cnu[dl[j]]) <= s->arena.n) words += cand_arena_words(cnu[dl[j++]]);
        CU_TRY(cudaMemcpyAsync(s->deferred.p, dl.data() + i, 4 * (j - i), cudaMemcpyHostToDevice, st));
        CU_TRY(cudaMemsetAsync(s->stats.p + 2, 0, 16, st));
        CandArgs cb = tmpl;
        cb.arena = s->arena.p;
        cb.arena_words = s->arena.n;
        cb.qlist = s->deferred.p;
        cb.nq = (int)(j - i);
        cb.deferred = s->deferred.p + (j - i);  // never written: the chunk fits
        CU_TRY(launch_candidates(cb, st));
        s->launches += 1;
        CU_TRY(cudaMemcpyAsync(s->h_stats.p, s->stats.p, 8 * 4, cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaStreamSynchronize(st));
        if ((s->h_stats.p[3] & 0xffffffffu) != 0) return fail(CULSH_ERR_DEVICE, "candidate admission failed");
        i = j;
    }
    return CULSH_OK;
}

// After the plan ran: waits for its statistics, re-runs the candidate stage
// per query when a work-stealing partition overflowed, and admits the
// queries whose candidate sets did not fit the arena in chunks
// (cuLSH_SearchTables.cu:282-306).
int finish_search(culsh_search* s, const SearchPlan& P, cudaStream_t st) {
    const int Q = P.Q;
    const CandArgs& ca = P.ca;
    CU_TRY(cudaStreamSynchronize(st));
    s->ws_used = P.use_ws;
    s->ws_overflow = 0;
    s->deferred_queries = 0;
    if (P.use_ws && (s->h_stats.p[4] >> 32) != 0) {
        // A partition overflowed the shared-memory set (or the plan outgrew the
        // partial-list buffers): redo the stage with the per-query kernel,
        // whose global arena takes any set size.
        s->ws_overflow = 1;
        CU_TRY(cudaMemsetAsync(s->stats.p, 0, 8 * kStatWords, st));
        CU_TRY(launch_candidates(ca, st));
        s->launches += 1;
        CU_TRY(cudaMemcpyAsync(s->h_stats.p, s->stats.p, 8 * kStatWords, cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaStreamSynchronize(st));
    }
    unsigned int ndef = (unsigned int)(s->h_stats.p[3] & 0xffffffffu);
    if (ndef) {
        std::vector<int> dl(ndef);
        CU_TRY(cudaMemcpyAsync(dl.data(), s->deferred.p, 4 * (size_t)ndef, cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaStreamSynchronize(st));
        s->deferred_queries = (int)ndef;
        TRY(rerun_queries(s, ca, std::move(dl), Q, st));
    }
    s->tot_unique = s->h_stats.p[0];
    s->tot_nonunique = s->h_stats.p[1];
    s->knn_queries = s->knn_fallback = s->bucket_rows = 0;
    if (P.use_knn && !s->ws_overflow) {
        if ((s->h_stats.p[11] & 0xffffffffu) != 0)
            return fail(CULSH_ERR_DEVICE, "tensor-core k-NN: a bounded device wait gave up");
        s->knn_queries = (int)(s->h_stats.p[7] & 0xffffffffu);
        s->bucket_rows = P.wa.nbig;
        // queries whose bound-form lists could not prove their top-K: the
        // exact per-query kernel (their counts were taken already)
        const unsigned int nfb = (unsigned int)(s->h_stats.p[10] & 0xffffffffu);
        if (nfb) {
            std::vector<int> fl(nfb);
            CU_TRY(cudaMemcpyAsync(fl.data(), s->kfallback.p, 4 * (size_t)nfb, cudaMemcpyDeviceToHost, st));
            CU_TRY(cudaStreamSynchronize(st));
            CandArgs cb = ca;
            cb.totals = s->stats.p + 12;
            TRY(rerun_queries(s, cb, std::move(fl), Q, st));
            s->knn_fallback = (int)nfb;
        }
    }
    s->rechecked = P.use_ws && P.wa.bf16 && !s->ws_overflow ? (long long)s->h_stats.p[6] : 0;
    s->dense_queries = P.use_ws && P.use_dense && !s->ws_overflow ? (int)(s->h_stats.p[7] & 0xffffffffu) : 0;
    return CULSH_OK;
}

// The query path on device buffers (cuLSH_SearchTables.cu:197-463). Planning
// (which may grow buffers) and graph capture hold the process-wide lock, so
// that searches on other threads (the serving loop's slots) never free device
// memory during a capture; launches and the wait for results do not.
int search_device(culsh_search* s, const float* dQ, int Q, int32_t* d_ids, float* d_d, cudaStream_t st,
                  const float* proj_src = nullptr) {
    SearchPlan P;
    {
        std::lock_guard<std::mutex> lk(alloc_capture_mutex());
        TRY(plan_search(s, dQ, Q, d_ids, d_d, st, &P, proj_src));
        s->last_stage_events = P.stage_events != 0;
        s->host_copy_timed = false;
        s->host_path = 0;
        TRY(run_plan(s, P, st));
    }
    return finish_search(s, P, st);
}

}  // namespace

// ============================================================================
extern "C" {

const char* culsh_last_error(void) { return g_err.c_str(); }
int culsh_version(void) { return 10000; }

int culsh_index_create(culsh_index** out) {
    if (!out) return fail(CULSH_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = new (std::nothrow) culsh_index();
    return *out ? CULSH_OK : fail(CULSH_ERR_OUT_OF_MEMORY, "host allocation failed");
}

void culsh_index_destroy(culsh_index* ix) { delete ix; }

static int reset_common(culsh_index* ix, int N, int D, int L, int M, float W) {
    if (!ix) return fail(CULSH_ERR_INVALID_ARGUMENT, "null index");
    TRY(check_params(N, D, L, M, W));
    clear_index_state(ix);
    ix->N = N;
    ix->D = D;
    ix->L = L;
    ix->M = M;
    ix->W = W;
    ix->A.assign((size_t)L * M * D, 0.0f);
    ix->b.assign((size_t)L * M, 0.0f);
    ix->has_proj = false;
    return CULSH_OK;
}

int culsh_index_reset_random(culsh_index* ix, int N, int D, int L, int M, float W, unsigned long long seed, FILE* dbg) {
    TRY(reset_common(ix, N, D, L, M, W));
    TRY(ensure_stream(&ix->stream));
    cudaStream_t st = ix->stream;
    const size_t nA = (size_t)L * M * D, nu = (size_t)L * M;
    DevBuf<float> dA, du;
    CU_TRY(dA.reserve(nA));
    CU_TRY(du.reserve(nu));
    CU_TRY(launch_random_projection(dA.p, du.p, (int64_t)nA, (int64_t)nu, seed, st));
    CU_TRY(cudaMemcpyAsync(ix->A.data(), dA.p, 4 * nA, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaMemcpyAsync(ix->b.data(), du.p, 4 * nu, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    // cuLSH_HashTables.cu:169-171: b = (u - min u) * W per table.
    for (int l = 0; l < L; ++l) {
        float* bl = ix->b.data() + (size_t)l * M;
        const float mn = *std::min_element(bl, bl + M);
        for (int m = 0; m < M; ++m) bl[m] = (bl[m] - mn) * W;
    }
    ix->has_proj = true;
    if (dbg)
        fprintf(dbg, "[HashTables::reset]\tIndexing structure reset with parameters (N, D, L, M, W) = (%d, %d, %d, %d, %.2f), and random matrices [A] & vectors [b].\n",
                N, D, L, M, W);
    return CULSH_OK;
}

int culsh_index_reset(culsh_index* ix, int N, int D, int L, int M, float W, const float* const* A,
                      const float* const* b, FILE* dbg) {
    TRY(reset_common(ix, N, D, L, M, W));
    if (!A || !b) return fail(CULSH_ERR_INVALID_ARGUMENT, "Pointers to matrices [A] and/or vectors [b] are null.");
    for (int l = 0; l < L; ++l) {
        if (!A[l] || !b[l]) return fail(CULSH_ERR_INVALID_ARGUMENT, "A[%d] or b[%d] is null", l, l);
        std::memcpy(ix->A.data() + (size_t)l * M * D, A[l], sizeof(float) * (size_t)M * D);
        std::memcpy(ix->b.data() + (size_t)l * M, b[l], sizeof(float) * M);
    }
    ix->has_proj = true;
    if (dbg)
        fprintf(dbg, "[HashTables::reset]\tIndexing structure reset with parameters (N, D, L, M, W) = (%d, %d, %d, %d, %.2f), matrices [A] & vectors [b] have been manually set.\n",
                N, D, L, M, W);
    return CULSH_OK;
}

static int precheck_build(culsh_index* ix) {
    if (!ix) return fail(CULSH_ERR_INVALID_ARGUMENT, "null index");
    if (!(ix->N > 0 && ix->D > 0 && ix->L > 0 && ix->M > 0 && ix->W > 0.0f))
        return fail(CULSH_ERR_STATE, "Parameters must be positive. Have you reset the index structure properly???");
    if (!ix->has_proj)
        return fail(CULSH_ERR_STATE,
                    "Pointers to projection matrices [A] and vectors [b] must be valid. Have you reset the index structure properly???");
    return CULSH_OK;
}

int culsh_index_build(culsh_index* ix, const float* X, FILE* dbg) {
    TRY(precheck_build(ix));
    if (!X) return fail(CULSH_ERR_INVALID_ARGUMENT, "null dataset");
    TRY(ensure_stream(&ix->stream));
    cudaStream_t st = ix->stream;
    clear_index_state(ix);
    CU_TRY(ix->X.reserve((size_t)ix->N * ix->D));
    CU_TRY(cudaMemcpyAsync(ix->X.p, X, sizeof(float) * (size_t)ix->N * ix->D, cudaMemcpyHostToDevice, st));
    ix->x_src = X;
    return build_device(ix, ix->X.p, st, dbg);
}

int culsh_index_build_device(culsh_index* ix, const float* d_X, void* stream) {
    TRY(precheck_build(ix));
    if (!d_X) return fail(CULSH_ERR_INVALID_ARGUMENT, "null dataset");
    TRY(ensure_stream(&ix->stream));
    cudaStream_t st = stream ? (cudaStream_t)stream : ix->stream;
    clear_index_state(ix);
    ix->x_borrow = d_X;
    const int rc = build_device(ix, d_X, st, nullptr);
    if (rc == CULSH_OK && stream) CU_TRY(cudaStreamSynchronize(st));
    return rc;
}

int culsh_index_save(culsh_index* ix, const char* path, FILE* dbg) {
    if (!ix || !path) return fail(CULSH_ERR_INVALID_ARGUMENT, "null argument");
    if (dbg) fprintf(dbg, "[HashTables::save]\tSaving indexing structure to file \"%s\"...\n", path);
    if (!ix->has_proj)
        return fail(CULSH_ERR_STATE, "Pointers to matrices [A] and/or vectors [b] are null. Have you reset the index structure properly???");
    if (!ix->indexed) return fail(CULSH_ERR_STATE, "Pointers to bucket objects are null. Have you performed indexing???");
    TRY(ensure_host(ix));
    FILE* fp = fopen(path, "wb");
    if (!fp)
        return fail(CULSH_ERR_IO, "Could not create file \"%s\" in order to store the hash tables...", path);
    // Layout of cuLSH_HashTables.cu:415-433.
    const int L = ix->L, M = ix->M, D = ix->D, N = ix->N;
    bool ok = fwrite(&ix->N, 4, 1, fp) == 1 && fwrite(&ix->D, 4, 1, fp) == 1 && fwrite(&ix->L, 4, 1, fp) == 1 &&
              fwrite(&ix->M, 4, 1, fp) == 1 && fwrite(&ix->W, 4, 1, fp) == 1;
    for (int l = 0; ok && l < L; ++l)
        ok = fwrite(ix->A.data() + (size_t)l * M * D, 4, (size_t)M * D, fp) == (size_t)M * D &&
             fwrite(ix->b.data() + (size_t)l * M, 4, M, fp) == (size_t)M;
    ok = ok && fwrite(ix->buckets.data(), 4, L, fp) == (size_t)L;
    for (int l = 0; ok && l < L; ++l) {
        const size_t B = ix->buckets[l];
        ok = fwrite(ix->h_ids[l].data(), 4, N, fp) == (size_t)N && fwrite(ix->h_starts[l].data(), 4, B, fp) == B &&
             fwrite(ix->h_sizes[l].data(), 4, B, fp) == B && fwrite(ix->h_codes[l].data(), 4, B * M, fp) == B * M;
    }
    ok = !ferror(fp) && ok;
    ok = (fclose(fp) == 0) && ok;
    if (!ok) return fail(CULSH_ERR_IO, "writing \"%s\" failed", path);
    return CULSH_OK;
}

int culsh_index_load(culsh_index* ix, const char* path, FILE* dbg) {
    if (!ix || !path) return fail(CULSH_ERR_INVALID_ARGUMENT, "null argument");
    if (dbg) fprintf(dbg, "[HashTables::reset]\tLoading indexing structure from file \"%s\"...\n", path);
    FILE* fp = fopen(path, "rb");
    if (!fp)
        return fail(CULSH_ERR_IO,
                    "Could not open file \"%s\" in order to load the hash tables, or file does not exist...", path);
    struct Closer {
        FILE* f;
        ~Closer() { fclose(f); }
    } closer{fp};
    int hdr[4];
    float W;
    if (fread(hdr, 4, 4, fp) != 4 || fread(&W, 4, 1, fp) != 1)
        return fail(CULSH_ERR_FORMAT, "\"%s\": truncated header", path);
    const int N = hdr[0], D = hdr[1], L = hdr[2], M = hdr[3];
    {
        const int rc = check_params(N, D, L, M, W);
        if (rc != CULSH_OK) return fail(CULSH_ERR_FORMAT, "\"%s\": %s", path, g_err.c_str());
    }
    // The file size must match the header before anything large is allocated.
    if (fseek(fp, 0, SEEK_END) != 0) return fail(CULSH_ERR_IO, "\"%s\": seek failed", path);
    const long long fsize = ftell(fp);
    const long long fixed = 20 + 4ll * L * ((long long)D * M + M) + 4ll * L + 4ll * L * N;
    if (fsize < fixed) return fail(CULSH_ERR_FORMAT, "\"%s\": file is truncated (%lld < %lld bytes)", path, fsize, fixed);
    fseek(fp, 20, SEEK_SET);
    TRY(reset_common(ix, N, D, L, M, W));
    for (int l = 0; l < L; ++l) {
        if (fread(ix->A.data() + (size_t)l * M * D, 4, (size_t)M * D, fp) != (size_t)M * D ||
            fread(ix->b.data() + (size_t)l * M, 4, M, fp) != (size_t)M)
            return fail(CULSH_ERR_FORMAT, "\"%s\": truncated projection", path);
    }
    ix->has_proj = true;
    ix->buckets.assign(L, 0);
    if (fread(ix->buckets.data(), 4, L, fp) != (size_t)L) return fail(CULSH_ERR_FORMAT, "\"%s\": truncated bucket counts", path);
    long long expect = fixed;
    for (int l = 0; l < L; ++l) {
        if (ix->buckets[l] == 0 || ix->buckets[l] > (unsigned)N)
            return fail(CULSH_ERR_FORMAT, "\"%s\": table %d has %u buckets for %d points", path, l, ix->buckets[l], N);
        expect += 4ll * ix->buckets[l] * (2 + M);
    }
    if (fsize != expect) return fail(CULSH_ERR_FORMAT, "\"%s\": size %lld does not match its header (%lld)", path, fsize, expect);
    ix->h_ids.assign(L, {});
    ix->h_starts.assign(L, {});
    ix->h_sizes.assign(L, {});
    ix->h_codes.assign(L, {});
    for (int l = 0; l < L; ++l) {
        const size_t B = ix->buckets[l];
        ix->h_ids[l].resize(N);
        ix->h_starts[l].resize(B);
        ix->h_sizes[l].resize(B);
        ix->h_codes[l].resize(B * M);
        if (fread(ix->h_ids[l].data(), 4, N, fp) != (size_t)N || fread(ix->h_starts[l].data(), 4, B, fp) != B ||
            fread(ix->h_sizes[l].data(), 4, B, fp) != B || fread(ix->h_codes[l].data(), 4, B * M, fp) != B * M)
            return fail(CULSH_ERR_FORMAT, "\"%s\": truncated table %d", path, l);
        // Consistency: buckets tile [0, N) in order and ids are in range.
        uint64_t pos = 0;
        for (size_t j = 0; j < B; ++j) {
            if (ix->h_starts[l][j] != pos || ix->h_sizes[l][j] == 0)
                return fail(CULSH_ERR_FORMAT, "\"%s\": table %d bucket %zu is inconsistent", path, l, j);
            pos += ix->h_sizes[l][j];
        }
        if (pos != (uint64_t)N) return fail(CULSH_ERR_FORMAT, "\"%s\": table %d buckets cover %llu of %d points", path, l,
                                            (unsigned long long)pos, N);
        for (int i = 0; i < N; ++i)
            if (ix->h_ids[l][i] >= (unsigned)N) return fail(CULSH_ERR_FORMAT, "\"%s\": table %d id out of range", path, l);
    }
    ix->indexed = ix->host_valid = true;
    ix->dev_valid = false;
    ix->xb_valid = false;
    ix->kx_valid = false;
    if (dbg)
        fprintf(dbg, "[HashTables::load]\tIndexing structure loaded from file \"%s\", (N, D, L, M, W) = (%d, %d, %d, %d, %.2f)\n",
                path, N, D, L, M, W);
    return CULSH_OK;
}

}  // extern "C"

// Makes the index and its dataset device-resident (serving loop start-up), so
// that concurrent searches only read it.
int culsh::index_make_resident(culsh_index* ix) {
    if (!ix) return fail(CULSH_ERR_INVALID_ARGUMENT, "null index");
    if (!ix->indexed && !ix->host_valid) return fail(CULSH_ERR_STATE, "No index: have you performed indexing or loaded a file???");
    if (!ix->dev_x())
        return fail(CULSH_ERR_STATE, "the dataset is not on the device (index it, or search once with it after a load)");
    TRY(ensure_stream(&ix->stream));
    TRY(ensure_device(ix, ix->stream));
    CU_TRY(cudaStreamSynchronize(ix->stream));
    return CULSH_OK;
}

extern "C" {

void culsh_index_params(const culsh_index* ix, int* N, int* D, int* L, int* M, float* W) {
    if (N) *N = ix ? ix->N : 0;
    if (D) *D = ix ? ix->D : 0;
    if (L) *L = ix ? ix->L : 0;
    if (M) *M = ix ? ix->M : 0;
    if (W) *W = ix ? ix->W : 0.0f;
}

const float* culsh_index_A(culsh_index* ix, int table) {
    if (!ix || !ix->has_proj || table < 0 || table >= ix->L) return nullptr;
    return ix->A.data() + (size_t)table * ix->M * ix->D;
}
const float* culsh_index_b(culsh_index* ix, int table) {
    if (!ix || !ix->has_proj || table < 0 || table >= ix->L) return nullptr;
    return ix->b.data() + (size_t)table * ix->M;
}
unsigned culsh_index_bucket_count(culsh_index* ix, int table) {
    if (!ix || !ix->indexed || table < 0 || table >= ix->L) return 0;
    return ix->buckets[table];
}
const unsigned* culsh_index_bucket_counts(culsh_index* ix) {
    if (!ix || !ix->indexed) return nullptr;
    return ix->buckets.data();
}
#define HOST_GETTER(name, member)                                                     \
    if (!ix || !ix->indexed || table < 0 || table >= ix->L) return nullptr;           \
    if (ensure_host(ix) != CULSH_OK) return nullptr;                                  \
    return ix->member[table].data();
const unsigned* culsh_index_total_indices(culsh_index* ix, int table) { HOST_GETTER(total_indices, h_ids) }
const unsigned* culsh_index_starting_indices(culsh_index* ix, int table) { HOST_GETTER(starting_indices, h_starts) }
const unsigned* culsh_index_sizes(culsh_index* ix, int table) { HOST_GETTER(sizes, h_sizes) }
const float* culsh_index_codes(culsh_index* ix, int table) { HOST_GETTER(codes, h_codes) }
#undef HOST_GETTER

int culsh_index_profile_get(culsh_index* ix, culsh_index_profile* out) {
    if (!ix || !out) return fail(CULSH_ERR_INVALID_ARGUMENT, "null argument");
    *out = culsh_index_profile{};
    if (!ix->built_once) return fail(CULSH_ERR_STATE, "no index has been built on the device");
    CU_TRY(cudaEventSynchronize(ix->bev[4]));
    CU_TRY(cudaEventElapsedTime(&out->project_ms, ix->bev[0], ix->bev[1]));
    CU_TRY(cudaEventElapsedTime(&out->pack_ms, ix->bev[1], ix->bev[2]));
    CU_TRY(cudaEventElapsedTime(&out->sort_ms, ix->bev[2], ix->bev[3]));
    CU_TRY(cudaEventElapsedTime(&out->bucket_ms, ix->bev[3], ix->bev[4]));
    CU_TRY(cudaEventElapsedTime(&out->total_ms, ix->bev[0], ix->bev[4]));
    out->tensor_cores = ix->tc_recomputed >= 0;
    out->recomputed = ix->tc_recomputed;
    out->key_words = ix->KW;
    out->sort_passes = ix->sort_passes;
    out->sort_form = ix->sort_form;
    return CULSH_OK;
}

int culsh_search_create(culsh_search** out) {
    if (!out) return fail(CULSH_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = new (std::nothrow) culsh_search();
    return *out ? CULSH_OK : fail(CULSH_ERR_OUT_OF_MEMORY, "host allocation failed");
}

void culsh_search_destroy(culsh_search* s) { delete s; }

int culsh_search_reset(culsh_search* s, culsh_index* ix, int K, int T) {
    if (!s) return fail(CULSH_ERR_INVALID_ARGUMENT, "null search");
    s->ix = ix;
    s->L = ix ? ix->L : 0;
    s->K = K;
    s->T = T;
    s->Q = 0;
    s->searched = false;
    s->qb_host_valid = false;
    s->tot_unique = s->tot_nonunique = 0;
    s->times = culsh_times{};
    return CULSH_OK;
}

static int precheck_search(culsh_search* s, int Q) {
    if (!s) return fail(CULSH_ERR_INVALID_ARGUMENT, "null search");
    if (!s->ix) return fail(CULSH_ERR_STATE, "No indexing structure has been associated with searching structure...");
    if (Q <= 0 || s->L <= 0 || s->K <= 0 || s->T <= 0)
        return fail(CULSH_ERR_INVALID_ARGUMENT,
                    "Integer parameters must be all positive. Have you reset the indexing structure properly before assigning it to this searching structure???");
    if (s->L != s->ix->L) return fail(CULSH_ERR_STATE, "the index changed since SearchTables::reset");
    if (s->K > CULSH_MAX_K) return fail(CULSH_ERR_CAPACITY, "K = %d exceeds the supported maximum %d", s->K, CULSH_MAX_K);
    if (s->T > CULSH_MAX_T) return fail(CULSH_ERR_CAPACITY, "T = %d exceeds the supported maximum %d", s->T, CULSH_MAX_T);
    if (!s->ix->indexed) return fail(CULSH_ERR_STATE, "the index structure has not been indexed or loaded");
    return CULSH_OK;
}

// Whether kernels may read pageable host memory (Grace-Blackwell: through
// the host page tables over NVLink-C2C). CULSH_NO_DIRECT_HOST disables its use.
static bool direct_host_access() {
    static int v = -1;
    if (v < 0) {
        int dev = 0, a = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess)
            a = 0;
        v = a ? 1 : 0;
    }
    return v == 1 && getenv("CULSH_NO_DIRECT_HOST") == nullptr;
}

int culsh_search_run(culsh_search* s, const float* queries, int Q, const float* dataset, FILE* dbg) {
    TRY(precheck_search(s, Q));
    if (!queries) return fail(CULSH_ERR_INVALID_ARGUMENT, "null queries");
    culsh_index* ix = s->ix;
    TRY(ensure_stream(&s->stream));
    cudaStream_t st = s->stream;
    s->searched = false;
    s->qb_host_valid = false;
    const double t0 = seconds_now();
    TRY(ensure_device(ix, st));
    if (dataset && !ix->x_borrow && !(ix->X.p && ix->x_src == dataset)) {
        CU_TRY(ix->X.reserve((size_t)ix->N * ix->D));
        CU_TRY(cudaMemcpyAsync(ix->X.p, dataset, sizeof(float) * (size_t)ix->N * ix->D, cudaMemcpyHostToDevice, st));
        ix->x_src = dataset;
        ix->xb_valid = false;
        ix->kx_valid = false;
    }
    if (!ix->dev_x()) return fail(CULSH_ERR_INVALID_ARGUMENT, "null dataset and no dataset on the device");
    const int D = ix->D, K = s->K;
    CU_TRY(s->h_ids.reserve((size_t)Q * K));
    CU_TRY(s->h_d.reserve((size_t)Q * K));
    if (dbg) fprintf(dbg, "[SearchTables::search]\tPerforming searching. (Q, K, T) = (%d, %d, %d)\n", Q, K, s->T);
    if (direct_host_access() && ((uintptr_t)queries & 15u) == 0) {
        // The kernels read the caller's (pageable) queries through the host
        // page tables (16-byte loads, hence the alignment condition) and the
        // search writes its results into the pinned result buffers: no
        // staging copies. With L*M <= 192 the projection reads the rows
        // itself and writes them to the device query buffer on the way, for
        // the candidate stage; otherwise a copy kernel does that first.
        CU_TRY(s->dq.reserve((size_t)Q * D));
        if (ix->L * ix->M <= 192 && getenv("CULSH_NO_FUSED_COPY") == nullptr) {
            TRY(search_device(s, s->dq.p, Q, s->h_ids.p, s->h_d.p, st, queries));
            s->host_path = 3;
        } else {
            CU_TRY(launch_copy_f32(queries, s->dq.p, (int64_t)Q * D, st));
            TRY(search_device(s, s->dq.p, Q, s->h_ids.p, s->h_d.p, st));
            s->host_path = 2;
        }
    } else {
        CU_TRY(s->dq.reserve((size_t)Q * D));
        CU_TRY(s->oids.reserve((size_t)Q * K));
        CU_TRY(s->od.reserve((size_t)Q * K));
        CU_TRY(cudaMemcpyAsync(s->dq.p, queries, sizeof(float) * (size_t)Q * D, cudaMemcpyHostToDevice, st));
        TRY(search_device(s, s->dq.p, Q, s->oids.p, s->od.p, st));
        CU_TRY(cudaMemcpyAsync(s->h_ids.p, s->oids.p, 4 * (size_t)Q * K, cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaMemcpyAsync(s->h_d.p, s->od.p, 4 * (size_t)Q * K, cudaMemcpyDeviceToHost, st));
        s->host_path = 1;
    }
    if (s->last_stage_events) CU_TRY(cudaEventRecord(s->ev[4], st));
    CU_TRY(cudaStreamSynchronize(st));
    s->host_copy_timed = true;
    float ms[3] = {0, 0, 0};
    if (s->last_stage_events) {
        cudaEventElapsedTime(&ms[0], s->ev[0], s->ev[2]);
        cudaEventElapsedTime(&ms[1], s->ev[2], s->ev[3]);
        cudaEventElapsedTime(&ms[2], s->ev[3], s->ev[4]);
    }
    s->times = culsh_times{ms[0] / 1e3f, 0.f, 0.f, 0.f, ms[1] / 1e3f, ms[2] / 1e3f};
    s->Q = Q;
    s->searched = true;
    if (dbg)
        fprintf(dbg, "[SearchTables::search]\tNon-unique: %llu, unique: %llu, selectivity: %.2f%% (%.3f ms)\n",
                s->tot_nonunique, s->tot_unique, culsh_search_selectivity(s) * 100.0, 1e3 * (seconds_now() - t0));
    return CULSH_OK;
}

int culsh_search_run_device(culsh_search* s, const float* d_queries, int Q, int* d_ids, float* d_dists, void* stream) {
    TRY(precheck_search(s, Q));
    if (!d_queries || !d_ids || !d_dists) return fail(CULSH_ERR_INVALID_ARGUMENT, "null device buffer");
    TRY(ensure_stream(&s->stream));
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    s->searched = false;
    s->qb_host_valid = false;
    TRY(ensure_device(s->ix, st));
    TRY(search_device(s, d_queries, Q, d_ids, d_dists, st));
    s->Q = Q;
    s->searched = false;   // results live in the caller's device buffers
    return CULSH_OK;
}

long long culsh_search_device_bytes(culsh_search* s) {
    if (!s) return 0;
    size_t b = 0;
    auto add = [&](const auto& buf) { b += buf.n * sizeof(*buf.p); };
    add(s->dq);
    add(s->vals);
    add(s->od);
    add(s->qb);
    add(s->ph);
    add(s->pmask);
    add(s->pctx);
    add(s->oids);
    add(s->cnu);
    add(s->cu);
    add(s->stats);
    add(s->deferred);
    add(s->arena);
    add(s->q_items);
    add(s->q_off);
    add(s->item_q);
    add(s->part_n);
    add(s->q_done);
    add(s->item_p);
    add(s->part_d);
    add(s->part_i);
    add(s->dense_q);
    add(s->qorder);
    add(s->qorder_bins);
    add(s->kbm);
    add(s->kq_h);
    add(s->kq_l);
    add(s->kq_sq);
    add(s->kq_base);
    add(s->kq_bound);
    add(s->kpart_key);
    add(s->kpart_id);
    add(s->kpart_n);
    add(s->kfallback);
    return (long long)b;
}

long long culsh_search_estimate_bytes(const culsh_index* ix, int Q, int K, int T) {
    if (!ix || Q <= 0 || K <= 0 || T <= 0) return 0;
    const size_t L = ix->L, M = ix->M, q = (size_t)Q, k = (size_t)K;
    size_t b = 4 * L * M * q + 4 * L * q * (size_t)T + 8 * q + 8 * q + 64 + 8 * q + 4 * kArenaInitialWords;
    const size_t per_item = k * 8 + 4 + 4 + 1;
    size_t cap = std::max<size_t>(2 * q, kWsPartialBytes / per_item);
    cap = std::min(cap, q * kWsPartitions);
    b += 16 * q + cap * per_item;   // per-query plan arrays, dense-query list, partial lists
    b += 4 * q + 4 * (kOrderBins + 1);   // locality order
    if (M <= 16) b += 12 * L * q * (size_t)T + 48 * L * q;   // split probe lookups
    if (ix->D <= 128 && K <= kMaxKnnK) {
        // tensor-core path for dense queries: membership rows, query rows,
        // partial lists (at most 160 CTAs' list sets plus one per query tile)
        const size_t qc = (q + 2 * kKnnTileQ - 1) / (2 * kKnnTileQ) * (2 * kKnnTileQ);
        const size_t dp = ((size_t)ix->D + 63) / 64 * 64;
        const size_t nwp = (((size_t)ix->N + 31) / 32 + 3) / 4 * 4;
        const size_t lists = (160 + qc / kKnnTileQ) * 2 * kKnnTileQ;
        const size_t bmb = 4 * qc * nwp;
        if (bmb <= kKnnMaxBitmapBytes) b += bmb + 4 * qc * dp + 12 * qc + lists * (4 + 8 * (size_t)kMaxKnnK);
    }
    return (long long)b;
}

int culsh_search_release(culsh_search* s) {
    if (!s) return fail(CULSH_ERR_INVALID_ARGUMENT, "null search");
    std::lock_guard<std::mutex> lk(alloc_capture_mutex());
    drop_graph(s);
    s->dq.release();
    s->vals.release();
    s->od.release();
    s->qb.release();
    s->ph.release();
    s->pmask.release();
    s->pctx.release();
    s->oids.release();
    s->cnu.release();
    s->cu.release();
    s->stats.release();
    s->deferred.release();
    s->arena.release();
    s->q_items.release();
    s->q_off.release();
    s->item_q.release();
    s->part_n.release();
    s->q_done.release();
    s->item_p.release();
    s->part_d.release();
    s->part_i.release();
    s->dense_q.release();
    s->qorder.release();
    s->qorder_bins.release();
    s->kbm.release();
    s->kq_h.release();
    s->kq_l.release();
    s->kq_sq.release();
    s->kq_base.release();
    s->kq_bound.release();
    s->kpart_key.release();
    s->kpart_id.release();
    s->kpart_n.release();
    s->kfallback.release();
    s->Q = 0;
    s->searched = false;
    s->qb_host_valid = false;
    return CULSH_OK;
}

static void tune_to_c(const SearchTune& t, culsh_tuning* o) {
    o->proj_tile = t.proj_tile;
    o->probe_batch = t.probe_pch;
    o->candidates_mode = t.cand_ws;
    o->ws_threads = t.ws_wt;
    o->ws_blocks_per_sm = t.ws_bps;
    o->ws_chunk = t.ws_chunk;
    o->distance_bf16 = t.dist_bf16;
    o->ws_set_slots = t.ws_slots;
    o->probe_split = t.probe_split;
    o->ws_order = t.ws_order;
    o->dense_tc = t.dense_tc;
    o->dense_min = t.dense_min;
}

int culsh_search_get_tuning(culsh_search* s, culsh_tuning* out) {
    if (!s || !out) return fail(CULSH_ERR_INVALID_ARGUMENT, "null argument");
    *out = culsh_tuning{};
    tune_to_c(s->tune, out);
    return CULSH_OK;
}

int culsh_search_set_tuning(culsh_search* s, const culsh_tuning* in) {
    if (!s || !in) return fail(CULSH_ERR_INVALID_ARGUMENT, "null argument");
    const bool ok = in->proj_tile >= 0 && in->proj_tile <= 4 &&
                    (in->probe_batch == 1 || in->probe_batch == 2 || in->probe_batch == 4) &&
                    (in->candidates_mode == 0 || in->candidates_mode == 1) &&
                    (in->ws_threads == 64 || in->ws_threads == 128 || in->ws_threads == 256 ||
                     in->ws_threads == 512) &&
                    in->ws_blocks_per_sm >= 0 && in->ws_blocks_per_sm <= 64 && in->ws_chunk >= 64 &&
                    in->ws_chunk <= 65536 && (in->distance_bf16 == 0 || in->distance_bf16 == 1) &&
                    (in->ws_set_slots == 4096 || in->ws_set_slots == 8192 || in->ws_set_slots == 16384) &&
                    in->probe_split >= 0 && in->probe_split <= 2 && (in->ws_order == 0 || in->ws_order == 1) &&
                    (in->dense_tc == 0 || in->dense_tc == 1) && in->dense_min >= 0;
    if (!ok) return fail(CULSH_ERR_INVALID_ARGUMENT, "tuning value out of range");
    s->tune.proj_tile = in->proj_tile;
    s->tune.probe_pch = in->probe_batch;
    s->tune.cand_ws = in->candidates_mode;
    s->tune.ws_wt = in->ws_threads;
    s->tune.ws_bps = in->ws_blocks_per_sm;
    s->tune.ws_chunk = in->ws_chunk;
    s->tune.dist_bf16 = in->distance_bf16;
    s->tune.ws_slots = in->ws_set_slots;
    s->tune.probe_split = in->probe_split;
    s->tune.ws_order = in->ws_order;
    s->tune.dense_tc = in->dense_tc;
    s->tune.dense_min = in->dense_min;
    return CULSH_OK;
}

int culsh_search_set_graphs(culsh_search* s, int enabled) {
    if (!s) return fail(CULSH_ERR_INVALID_ARGUMENT, "null search");
    s->use_graphs = enabled != 0;
    return CULSH_OK;
}

int culsh_search_set_profiling(culsh_search* s, int stage_times) {
    if (!s) return fail(CULSH_ERR_INVALID_ARGUMENT, "null search");
    s->stage_events = stage_times != 0;
    return CULSH_OK;
}

// Coordinate search: the projection tiling by its stage time, the probe form
// by its stage time, then the candidate stage over its kernel form, item
// width, set size and partition size, distance form and locality order
// jointly, then the residency. Each configuration is searched once untimed
// and three times timed (median of each stage, device events).
int culsh_search_autotune(culsh_search* s, const float* d_queries, int Q, int* d_ids, float* d_dists, void* stream,
                          culsh_tuning* out) {
    TRY(precheck_search(s, Q));
    if (!d_queries || !d_ids || !d_dists) return fail(CULSH_ERR_INVALID_ARGUMENT, "null device buffer");
    TRY(ensure_stream(&s->stream));
    cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    s->searched = false;
    s->qb_host_valid = false;
    TRY(ensure_device(s->ix, st));
    // the tuner times stages: stage events on while it runs, as before after
    struct EventsOn {
        culsh_search* s;
        bool was;
        ~EventsOn() { s->stage_events = was; }
    } events_on{s, s->stage_events};
    s->stage_events = true;
    const size_t nout = (size_t)Q * s->K;
    std::vector<int> ref_ids(nout), got_ids(nout);
    std::vector<float> ref_d(nout), got_d(nout);
    unsigned long long ref_u = 0, ref_nu = 0;
    bool have_ref = false;
    int tried = 0;
    auto median3 = [](float a, float b, float c) { return std::max(std::min(a, b), std::min(std::max(a, b), c)); };
    // stage[0..2]: project, probe, candidates; stage[3]: whole search
    auto measure = [&](float stage[4]) -> int {
        float v[4][3];
        for (int r = -1; r < 3; ++r) {
            TRY(search_device(s, d_queries, Q, d_ids, d_dists, st));
            if (r < 0) continue;
            CU_TRY(cudaEventElapsedTime(&v[0][r], s->ev[0], s->ev[1]));
            CU_TRY(cudaEventElapsedTime(&v[1][r], s->ev[1], s->ev[2]));
            CU_TRY(cudaEventElapsedTime(&v[2][r], s->ev[2], s->ev[3]));
            CU_TRY(cudaEventElapsedTime(&v[3][r], s->ev[0], s->ev[3]));
        }
        for (int k = 0; k < 4; ++k) stage[k] = median3(v[k][0], v[k][1], v[k][2]);
        CU_TRY(cudaMemcpy(got_ids.data(), d_ids, 4 * nout, cudaMemcpyDeviceToHost));
        CU_TRY(cudaMemcpy(got_d.data(), d_dists, 4 * nout, cudaMemcpyDeviceToHost));
        if (!have_ref) {
            ref_ids = got_ids;
            ref_d = got_d;
            ref_u = s->tot_unique;
            ref_nu = s->tot_nonunique;
            have_ref = true;
        } else if (got_ids != ref_ids || std::memcmp(got_d.data(), ref_d.data(), 4 * nout) != 0 ||
                   s->tot_unique != ref_u || s->tot_nonunique != ref_nu) {
            return fail(CULSH_ERR_DEVICE, "autotune: configurations returned different results");
        }
        ++tried;
        return CULSH_OK;
    };
    const SearchTune start = s->tune;
    SearchTune best = start;
    float stage[4];
    float best_t = 0;
    // projection tiling
    for (int tile = 0; tile <= 4; ++tile) {
        s->tune = best;
        s->tune.proj_tile = tile;
        const int rc = measure(stage);
        if (rc != CULSH_OK) {
            s->tune = start;
            return rc;
        }
        if (tile == 0 || stage[0] < best_t) {
            best_t = stage[0];
            best.proj_tile = tile;
        }
    }
    // probe form: fused with batch depth 1, 2 or 4, or (M <= 16) split
    // lookups, or lookups at the end of the enumeration
    const int pchs[5] = {1, 2, 4, 0, -1};
    const int nforms = s->ix->M <= 16 ? 5 : 3;
    for (int i = 0; i < nforms; ++i) {
        s->tune = best;
        s->tune.probe_split = pchs[i] == 0 ? 1 : pchs[i] < 0 ? 2 : 0;
        if (pchs[i] > 0) s->tune.probe_pch = pchs[i];
        const int rc = measure(stage);
        if (rc != CULSH_OK) {
            s->tune = start;
            return rc;
        }
        if (i == 0 || stage[1] < best_t) {
            best_t = stage[1];
            best.probe_split = s->tune.probe_split;
            if (pchs[i] > 0) best.probe_pch = pchs[i];
        }
    }
    // candidate stage
    std::vector<SearchTune> cands;
    {
        SearchTune t = best;
        t.cand_ws = 0;
        cands.push_back(t);
        // (set slots, partition size): a partition of `chunk` non-unique
        // candidates always fits a set of 2 * chunk slots
        const int wts[4] = {64, 128, 256, 512};
        const int sets[7][2] = {{4096, 1024}, {4096, 2048}, {8192, 1024}, {8192, 2048},
                                {8192, 4096}, {16384, 4096}, {16384, 8192}};
        for (int o = 0; o < 2; ++o)
            for (int f = 0; f < 2; ++f)
                for (int a = 0; a < 4; ++a)
                    for (int b = 0; b < 7; ++b) {
                        SearchTune u = best;
                        u.cand_ws = 1;
                        u.ws_wt = wts[a];
                        u.ws_slots = sets[b][0];
                        u.ws_chunk = sets[b][1];
                        u.ws_bps = 0;
                        u.dist_bf16 = f;
                        u.ws_order = o;
                        cands.push_back(u);
                    }
    }
    bool first = true;
    for (const SearchTune& t : cands) {
        s->tune = t;
        const int rc = measure(stage);
        if (rc != CULSH_OK) {
            s->tune = start;
            return rc;
        }
        if (first || stage[2] < best_t) {
            best_t = stage[2];
            best = t;
            first = false;
        }
    }
    if (best.cand_ws) {   // residency: half the occupancy limit as well
        const int occ = ws_blocks_per_sm(s->ix->D, s->K, best.ws_wt, best.dist_bf16, best.ws_slots);
        if (occ > 1) {
            SearchTune t = best;
            t.ws_bps = occ / 2;
            s->tune = t;
            const int rc = measure(stage);
            if (rc != CULSH_OK) {
                s->tune = start;
                return rc;
            }
            if (stage[2] < best_t) {
                best = t;
                best_t = stage[2];
            }
        }
    }
    {
        // dense queries: tensor-core path or SIMT bitmap kernel, and (tensor
        // cores) the threshold from which a query is dense
        const unsigned long long N = (unsigned long long)s->ix->N;
        const int mins[3] = {0, (int)std::max(1024ull, N / 1024), (int)std::max(1024ull, N / 64)};
        const SearchTune base_t = best;
        float t_simt = -1.0f;   // the SIMT form (dense_tc = 0) at the chosen gather settings
        for (int tc = 0; tc < 2; ++tc)
            for (int mi = 0; mi < 3; ++mi) {
                if ((tc == 0 && mi > 0) || (tc == base_t.dense_tc && mins[mi] == base_t.dense_min)) continue;
                SearchTune t = base_t;
                t.dense_tc = tc;
                t.dense_min = mins[mi];
                s->tune = t;
                const int rc = measure(stage);
                if (rc != CULSH_OK) {
                    s->tune = start;
                    return rc;
                }
                if (tc == 0) t_simt = stage[2];
                if (stage[2] < best_t) {
                    best = t;
                    best_t = stage[2];
                }
            }
        if (base_t.dense_tc == 0) t_simt = best_t;
        // The gather settings above were chosen with the tensor-core path
        // taking the dense queries; without it every query is gathered and
        // another set and partition size may win. Where the SIMT form came
        // within 4x of the best, its item widths, set sizes, orders and
        // distance forms are tried again (the grid above, 112 configurations).
        if (best.dense_tc == 1 && best.cand_ws && t_simt > 0.0f && t_simt < 4.0f * best_t) {
            const int sets[7][2] = {{4096, 1024}, {4096, 2048}, {8192, 1024}, {8192, 2048},
                                    {8192, 4096}, {16384, 4096}, {16384, 8192}};
            const int wts[4] = {64, 128, 256, 512};
            const SearchTune simt_base = base_t;
            for (int f = 0; f < 2; ++f)
              for (int o = 0; o < 2; ++o)
               for (int w = 0; w < 4; ++w)
                for (int b = 0; b < 7; ++b) {
                    SearchTune t = simt_base;
                    t.dense_tc = 0;
                    t.dense_min = 0;
                    t.dist_bf16 = f;
                    t.ws_wt = wts[w];
                    t.ws_slots = sets[b][0];
                    t.ws_chunk = sets[b][1];
                    t.ws_order = o;
                    t.ws_bps = 0;
                    s->tune = t;
                    const int rc = measure(stage);
                    if (rc != CULSH_OK) {
                        s->tune = start;
                        return rc;
                    }
                    if (stage[2] < best_t) {
                        best = t;
                        best_t = stage[2];
                    }
                }
        }
    }
    s->tune = best;
    const int rc = measure(stage);
    if (rc != CULSH_OK) return rc;
    s->Q = Q;
    if (out) {
        *out = culsh_tuning{};
        tune_to_c(best, out);
        out->search_ms = stage[3];
        out->configs_tried = tried;
    }
    return CULSH_OK;
}

const int* culsh_search_knn_ids(culsh_search* s) { return (s && s->searched) ? s->h_ids.p : nullptr; }
const float* culsh_search_knn_distances(culsh_search* s) { return (s && s->searched) ? s->h_d.p : nullptr; }

const int* culsh_search_query_buckets(culsh_search* s, int table) {
    if (!s || !s->ix || s->Q <= 0 || table < 0 || table >= s->L || !s->qb.p) return nullptr;
    if (!s->qb_host_valid) {
        const size_t n = (size_t)s->L * s->Q * s->T;
        if (s->h_qb.reserve(n) != cudaSuccess) return nullptr;
        cudaStream_t st = s->stream;
        if (cudaMemcpyAsync(s->h_qb.p, s->qb.p, 4 * n, cudaMemcpyDeviceToHost, st) != cudaSuccess) return nullptr;
        if (cudaStreamSynchronize(st) != cudaSuccess) return nullptr;
        s->qb_host_valid = true;
    }
    return s->h_qb.p + (size_t)table * s->Q * s->T;
}

// cuLSH_SearchTables.cu:83: unique / N / Q.
float culsh_search_selectivity(culsh_search* s) {
    if (!s || !s->ix || !s->ix->N || !s->Q) return 0.0f;
    return (float)((double)s->tot_unique / (double)s->ix->N / (double)s->Q);
}
// cuLSH_SearchTables.cu:86: (nonUnique - unique) / unique.
float culsh_search_nonunique_percentage(culsh_search* s) {
    if (!s || !s->tot_unique) return 0.0f;
    return (float)((double)(s->tot_nonunique - s->tot_unique) / (double)s->tot_unique);
}
unsigned long long culsh_search_total_unique(culsh_search* s) { return s ? s->tot_unique : 0; }
unsigned long long culsh_search_total_nonunique(culsh_search* s) { return s ? s->tot_nonunique : 0; }
void culsh_search_times(culsh_search* s, culsh_times* out) {
    if (out) *out = s ? s->times : culsh_times{};
}

int culsh_search_profile_get(culsh_search* s, culsh_search_profile* out) {
    if (!s || !out) return fail(CULSH_ERR_INVALID_ARGUMENT, "null argument");
    *out = culsh_search_profile{};
    if (!s->ev[0] || s->Q <= 0) return fail(CULSH_ERR_STATE, "no search has run");
    out->stage_times = s->last_stage_events ? 1 : 0;
    if (s->last_stage_events) {
        CU_TRY(cudaEventSynchronize(s->ev[3]));
        CU_TRY(cudaEventElapsedTime(&out->project_ms, s->ev[0], s->ev[1]));
        CU_TRY(cudaEventElapsedTime(&out->probe_ms, s->ev[1], s->ev[2]));
        CU_TRY(cudaEventElapsedTime(&out->candidates_ms, s->ev[2], s->ev[3]));
        if (s->knn_queries > 0) {
            CU_TRY(cudaEventElapsedTime(&out->membership_ms, s->ev[2], s->ev[5]));
            CU_TRY(cudaEventElapsedTime(&out->knn_ms, s->ev[5], s->ev[3]));
        }
    }
    out->launches = s->launches;
    out->deferred_queries = s->deferred_queries;
    out->key_words = s->ix ? s->ix->KW : 0;
    out->candidates_mode = s->ws_used ? (s->ws_overflow ? 2 : 1) : 0;
    out->graph_mode = s->graph_mode;
    out->rechecked = s->rechecked;
    out->dense_queries = s->dense_queries;
    out->host_path = s->host_path;
    out->knn_queries = s->knn_queries;
    out->knn_fallback = s->knn_fallback;
    out->bucket_rows = s->bucket_rows;
    return CULSH_OK;
}

}  // extern "C"

// ============================================================================
// Search without any allocation.
//
// Some callers cannot call cudaMalloc: code running under a memory pool or
// arena they do not own, frameworks that forbid allocation inside a timed or
// latency-critical request path, and processes whose allocator is locked down
// after start-up. culsh_search_run_device_noalloc runs the same three kernels
// as culsh_search_run_device, but every scratch buffer (query projections,
// probe buckets, candidate counts, the overflow hash arena) is carved out of
// the fixed array below instead of being allocated.
//
// The array is reserved on every GPU that loads this library and is held
// until the process exits. Its address is looked up once per device, on the
// first call made with that device current (call it once before any stream
// capture). The index must already be resident on the device, and the call
// leaves the search object's getters (statistics, query buckets) describing
// its last ordinary search. All calls share the array and it keeps the previous call's
// contents: the counters that must start at zero are cleared by each call,
// and calls that overlap on the GPU (different streams, threads or
// processes-in-the-same-context) race on it and must be serialised by the
// caller.
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;   // 64 MiB
constexpr size_t kNoAllocMinArenaBytes = size_t(1) << 20;   // at least 1 MiB of overflow arena
constexpr int kNoAllocMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[kNoAllocMaxDevices] = {};

inline size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

int noalloc_scratch(unsigned char** out) {
    int dev = 0;
    CU_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(CULSH_ERR_CAPACITY, "device %d beyond %d", dev, kNoAllocMaxDevices);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        CU_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return CULSH_OK;
}

}  // namespace

extern "C" int culsh_search_run_device_noalloc(culsh_search* s, const float* d_queries, int Q, int* d_ids,
                                               float* d_dists, void* stream) {
    TRY(precheck_search(s, Q));
    if (!d_queries || !d_ids || !d_dists) return fail(CULSH_ERR_INVALID_ARGUMENT, "null device buffer");
    culsh_index* ix = s->ix;
    if (!ix->dev_valid || !ix->proj_on_dev || !ix->dev_x())
        return fail(CULSH_ERR_STATE,
                    "the index is not resident on the device: build it with index()/culsh_index_build_device, "
                    "or run one ordinary search after load(), before calling the no-allocation search");
    const cudaStream_t st = (cudaStream_t)stream;
    const int L = ix->L, M = ix->M, D = ix->D, K = s->K, T = s->T;
    // Layout of the fixed scratch for this call.
    size_t off = 0;
    const size_t o_vals = off;
    off = align256(off + sizeof(float) * (size_t)L * M * Q);
    const size_t o_qb = off;
    off = align256(off + sizeof(int32_t) * (size_t)L * Q * T);
    const size_t o_cnu = off;
    off = align256(off + 8 * (size_t)Q);
    const size_t o_cu = off;
    off = align256(off + 8 * (size_t)Q);
    const size_t o_stats = off;
    off = align256(off + 8 * 4);
    const size_t o_def = off;
    off = align256(off + sizeof(int) * 2 * (size_t)Q);
    const size_t o_arena = off;
    if (off + kNoAllocMinArenaBytes > kNoAllocScratchBytes)
        return fail(CULSH_ERR_CAPACITY,
                    "no-allocation search of Q=%d (L=%d, M=%d, T=%d) needs %zu bytes of scratch plus a 1 MiB "
                    "arena; the static scratch holds %zu bytes",
                    Q, L, M, T, off, kNoAllocScratchBytes);
    unsigned char* base = nullptr;
    TRY(noalloc_scratch(&base));
    float* vals = reinterpret_cast<float*>(base + o_vals);
    int32_t* qb = reinterpret_cast<int32_t*>(base + o_qb);
    unsigned long long* cnu = reinterpret_cast<unsigned long long*>(base + o_cnu);
    unsigned long long* cu = reinterpret_cast<unsigned long long*>(base + o_cu);
    unsigned long long* stats = reinterpret_cast<unsigned long long*>(base + o_stats);
    int* deferred = reinterpret_cast<int*>(base + o_def);
    uint32_t* arena = reinterpret_cast<uint32_t*>(base + o_arena);
    unsigned long long arena_words = (kNoAllocScratchBytes - o_arena) / 4;
    // CULSH_NOALLOC_ARENA_WORDS lowers the overflow arena below what the
    // fixed array leaves for it (never raises it); the tests use it to reach
    // the deferred rounds and the capacity error with small cases.
    if (const char* e = getenv("CULSH_NOALLOC_ARENA_WORDS"))
        arena_words = std::min<unsigned long long>(arena_words, std::max(1ll, atoll(e)));

    CU_TRY(cudaMemsetAsync(cnu, 0, 8 * (size_t)Q, st));
    CU_TRY(cudaMemsetAsync(stats, 0, 8 * 4, st));
    CU_TRY(launch_project_fp32(d_queries, Q, D, ix->dAT.p, ix->lmp, ix->db.p, L * M, ix->W, nullptr, vals, nullptr,
                               nullptr, nullptr, st));
    ProbeArgs pa{};
    pa.vals = vals;
    pa.Q = Q;
    pa.T = T;
    pa.lv = lookup_view(ix);
    pa.qbuckets = qb;
    pa.cnu = cnu;
    pa.small_codes = small_codes(ix);
    pa.pch = 2;
    CU_TRY(launch_probe(pa, st));
    CandArgs ca{};
    ca.X = ix->dev_x();
    ca.N = ix->N;
    ca.D = D;
    ca.L = L;
    ca.T = T;
    ca.Q = Q;
    ca.K = K;
    ca.queries = d_queries;
    ca.qbuckets = qb;
    ca.boff = ix->boff.p;
    ca.starts = ix->starts.p;
    ca.sizes = ix->sizes.p;
    ca.ids = ix->ids.p;
    ca.cnu = cnu;
    ca.out_ids = d_ids;
    ca.out_d = d_dists;
    ca.cu = cu;
    ca.totals = stats;
    ca.arena = arena;
    ca.arena_words = arena_words;
    ca.arena_top = stats + 2;
    ca.deferred = deferred;
    ca.n_deferred = reinterpret_cast<unsigned int*>(stats + 3);
    ca.qlist = nullptr;
    ca.nq = Q;
    CU_TRY(launch_candidates(ca, st));
    unsigned long long h_stats[4] = {0, 0, 0, 0};
    CU_TRY(cudaMemcpyAsync(h_stats, stats, sizeof h_stats, cudaMemcpyDeviceToHost, st));
    CU_TRY(cudaStreamSynchronize(st));
    // Queries whose candidate sets did not fit the arena at once are re-run
    // in rounds over the same arena; a round that admits nothing means one
    // query alone needs more than the arena.
    unsigned int ndef = (unsigned int)(h_stats[3] & 0xffffffffu);
    int cur = 0;
    while (ndef) {
        const unsigned int before = ndef;
        CandArgs cb = ca;
        cb.qlist = deferred + (size_t)cur * Q;
        cb.nq = (int)ndef;
        cb.deferred = deferred + (size_t)(cur ^ 1) * Q;
        CU_TRY(cudaMemsetAsync(stats + 2, 0, 16, st));
        CU_TRY(launch_candidates(cb, st));
        CU_TRY(cudaMemcpyAsync(h_stats, stats, sizeof h_stats, cudaMemcpyDeviceToHost, st));
        CU_TRY(cudaStreamSynchronize(st));
        ndef = (unsigned int)(h_stats[3] & 0xffffffffu);
        cur ^= 1;
        if (ndef == before)
            return fail(CULSH_ERR_CAPACITY,
                        "a query's candidate set needs more than the %llu-byte overflow arena of the static scratch",
                        arena_words * 4);
    }
    // The search object's getters keep describing its last ordinary search:
    // this call reports only through the caller's buffers.
    return CULSH_OK;
}
