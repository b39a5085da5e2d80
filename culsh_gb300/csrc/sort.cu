// K2 + K3: bucketing of the projected codes.
//
// Replaces cuLSH_Indexing.cu:71-93 (radixSortRows_1matrix: M gather + stable
// sort passes over float columns, per table) and cuLSH_Indexing.cu:98-169
// (calculateBuckets / copyMatrixRows: boundary flags, counts, unique codes).
//
// Each point's code row of table l is packed into a multi-word key: column m
// becomes a field of bit width fbits[l*M+m] (enough for cmax - cmin), column 0
// in the most significant bits, so unsigned key order equals the reference's
// lexicographic order on (c0, c1, ..., c_{M-1}). All L tables are sorted in
// one onesweep LSD radix sort (8-bit digits, decoupled look-back, one launch
// per digit pass over all tables); the sort is stable and starts from id
// order, so ids inside a bucket ascend as in the reference. A run-length pass
// then emits bucket starts, sizes and unique keys, and an open-addressing hash
// over the unique keys serves exact-code lookups at query time.
//
// Every pass streams keys and ids once in and once out (the digit's own
// word is read once): HBM bound.
#include <algorithm>
#include <climits>

#include "culsh_internal.cuh"

namespace culsh {
namespace {

constexpr int NT = 256;
constexpr int SP_ITEMS = 16;
constexpr int SP_TILE = NT * SP_ITEMS;      // 4096 elements per tile
constexpr int SP_WARPS = NT / 32;
constexpr uint32_t ST_AGG = 1u << 30;       // tile aggregate published
constexpr uint32_t ST_PRE = 2u << 30;       // inclusive prefix published
constexpr uint32_t ST_CNT = (1u << 30) - 1;
constexpr int HIST_CHUNK = 8192;
constexpr uint32_t kSpinLimit = 1u << 22;
constexpr int kRunMax = 2048;               // longest run of equal top words ordered in shared memory

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Exclusive scan of one value per thread over a 256-thread block.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* ws, uint32_t* total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = lane < SP_WARPS ? ws[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < SP_WARPS) ws[lane] = t;
    }
    __syncthreads();
    const uint32_t pre = w > 0 ? ws[w - 1] : 0;
    if (total) *total = ws[SP_WARPS - 1];
    const uint32_t r = pre + x - v;
    __syncthreads();
    return r;
}

__global__ void k_pack_keys(const int32_t* __restrict__ codes, int64_t N, int L, int M, int KW,
                            const int32_t* __restrict__ cmin, const uint8_t* __restrict__ fbits,
                            const uint16_t* __restrict__ foff, uint32_t* __restrict__ keys,
                            uint32_t* __restrict__ vals) {
    const int64_t LN = (int64_t)L * N;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < LN;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int l = (int)(idx / N);
        const int64_t n = idx - (int64_t)l * N;
        // fields are contiguous, column M - 1 at bit 0 and column 0 on top:
        // shift each column in after the previous one (registers only)
        unsigned __int128 kk = 0;
        for (int m = 0; m < M; ++m) {
            const int c = l * M + m;
            const int bits = __ldg(fbits + c);
            if (!bits) continue;
            kk = (kk << bits) | (uint32_t)(codes[(int64_t)c * N + n] - __ldg(cmin + c));
        }
#pragma unroll
        for (int w = 0; w < kMaxKW; ++w)
            if (w < KW) keys[w * LN + idx] = (uint32_t)(kk >> (32 * w));
        vals[idx] = (uint32_t)n;
    }
}

__global__ void k_sort_hist(const uint32_t* __restrict__ keys, int64_t N, int L, int passes,
                            uint32_t* __restrict__ hist) {
    extern __shared__ uint32_t sh[];
    for (int i = threadIdx.x; i < passes * 256; i += NT) sh[i] = 0;
    __syncthreads();
    const int l = blockIdx.y;
    const int64_t LN = (int64_t)L * N, seg = (int64_t)l * N;
    const int64_t start = (int64_t)blockIdx.x * HIST_CHUNK;
    const int64_t end = min(N, start + HIST_CHUNK);
    for (int w = 0; w * 4 < passes; ++w) {
        const uint32_t* kw = keys + w * LN + seg;
        const int np = min(4, passes - 4 * w);
        for (int64_t i = start + threadIdx.x; i < end; i += NT) {
            const uint32_t k = kw[i];
            for (int s = 0; s < np; ++s) atomicAdd(&sh[(4 * w + s) * 256 + ((k >> (8 * s)) & 255u)], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += NT)
        if (sh[i]) atomicAdd(&hist[(int64_t)l * passes * 256 + i], sh[i]);
}

__global__ void k_sort_digit_base(const uint32_t* __restrict__ hist, uint32_t* __restrict__ base) {
    __shared__ uint32_t ws[SP_WARPS];
    const int64_t o = (int64_t)blockIdx.x * 256 + threadIdx.x;
    base[o] = block_excl_scan(hist[o], ws, nullptr);
}

// One LSD digit pass over all tables. Tiles are taken in launch order from a
// global counter, so every tile's predecessors have started before it and the
// look-back wait always ends; it is bounded anyway (kErrSpin).
__global__ void __launch_bounds__(NT, 3) k_sort_pass(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                  uint32_t* __restrict__ kout, uint32_t* __restrict__ vout,
                                                  int64_t N, int L, int KW, int tiles, int word, int shift,
                                                  const uint32_t* __restrict__ base, int passes, int pass,
                                                  uint32_t* status, uint32_t* counter, int* err) {
    __shared__ uint32_t whist[SP_WARPS][256];
    __shared__ uint32_t tstart[256];
    __shared__ uint32_t gadd[256];
    __shared__ uint32_t buf[SP_TILE];
    __shared__ uint32_t wtile[SP_TILE];
    __shared__ uint8_t sdig[SP_TILE];
    __shared__ uint32_t ws[SP_WARPS];
    __shared__ uint32_t s_vb;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_vb = atomicAdd(counter, 1u);
    for (int i = tid; i < SP_WARPS * 256; i += NT) (&whist[0][0])[i] = 0;
    __syncthreads();
    const uint32_t vb = s_vb;
    const int l = (int)(vb / (uint32_t)tiles), tile = (int)(vb % (uint32_t)tiles);
    const int64_t LN = (int64_t)L * N, seg = (int64_t)l * N;
    const int64_t t0 = (int64_t)tile * SP_TILE;
    const int nvalid = (N - t0 < SP_TILE) ? (int)(N - t0) : SP_TILE;
    const uint32_t* kw = kin + word * LN + seg + t0;

    uint32_t dig[SP_ITEMS], pos[SP_ITEMS];
#pragma unroll
    for (int i = 0; i < SP_ITEMS; ++i) {
        const int e = warp * (32 * SP_ITEMS) + i * 32 + lane;
        const uint32_t w = (e < nvalid) ? kw[e] : 0u;
        wtile[e] = w;   // the digit's key word, kept for its own scatter
        dig[i] = (e < nvalid) ? ((w >> shift) & 255u) : 256u;
    }
    // Stable warp-level ranking: element order inside a warp chunk is
    // (item, lane), which is the element order of the tile.
#pragma unroll
    for (int i = 0; i < SP_ITEMS; ++i) {
        const uint32_t d = dig[i];
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        const uint32_t below = __popc(peers & ((1u << lane) - 1u));
        uint32_t cnt = 0;
        if (d < 256) cnt = whist[warp][d];
        __syncwarp();
        if (d < 256 && lane == leader) whist[warp][d] = cnt + __popc(peers);
        __syncwarp();
        pos[i] = cnt + below;
    }
    __syncthreads();
    // Thread tid owns digit tid: per-warp exclusive offsets and tile total.
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < SP_WARPS; ++w) {
        const uint32_t c = whist[w][tid];
        whist[w][tid] = run;
        run += c;
    }
    const uint32_t total = run;
    tstart[tid] = block_excl_scan(total, ws, nullptr);

    // Decoupled look-back for digit tid.
    uint32_t* my = status + ((int64_t)l * tiles + tile) * 256 + tid;
    uint32_t excl = 0;
    if (tile == 0) {
        st_relaxed(my, ST_PRE | total);
    } else {
        st_relaxed(my, ST_AGG | total);
        int j = tile - 1;
        uint32_t spins = 0;
        while (j >= 0) {
            const uint32_t s = ld_relaxed(status + ((int64_t)l * tiles + j) * 256 + tid);
            const uint32_t flag = s & ~ST_CNT;
            if (flag == 0) {
                if (++spins > kSpinLimit) {
                    atomicOr(err, kErrSpin);
                    break;
                }
                if ((spins & 31u) == 0) __nanosleep(64);
                continue;
            }
            excl += s & ST_CNT;
            if (flag == ST_PRE) break;
            --j;
        }
        st_relaxed(my, ST_PRE | (excl + total));
    }
    gadd[tid] = base[((int64_t)l * passes + pass) * 256 + tid] + excl - tstart[tid];
    __syncthreads();

#pragma unroll
    for (int i = 0; i < SP_ITEMS; ++i) {
        const uint32_t d = dig[i];
        if (d < 256) {
            pos[i] += tstart[d] + whist[warp][d];
            sdig[pos[i]] = (uint8_t)d;
        }
    }
    __syncthreads();
    // Global destination of tile position s = tid + k * NT (digit runs are
    // contiguous), computed once for all components.
    uint32_t doff[SP_ITEMS];
#pragma unroll
    for (int k = 0; k < SP_ITEMS; ++k) {
        const int sp = tid + k * NT;
        doff[k] = sp < nvalid ? gadd[sdig[sp]] + (uint32_t)sp : 0u;
    }
    // Scatter each component (ids, then key words) through shared memory so
    // that the global writes of one digit run are contiguous; the next
    // component's loads are issued before the current one is written out.
    auto load_comp = [&](int comp, uint32_t (&v)[SP_ITEMS]) {
        const uint32_t* src = (comp == 0 ? vin : kin + (comp - 1) * LN) + seg + t0;
#pragma unroll
        for (int i = 0; i < SP_ITEMS; ++i) {
            const int e = warp * (32 * SP_ITEMS) + i * 32 + lane;
            // the digit's own word is already in shared memory
            v[i] = dig[i] < 256 ? (comp == word + 1 ? wtile[e] : src[e]) : 0u;
        }
    };
    uint32_t cur[SP_ITEMS];
    load_comp(0, cur);
    for (int comp = 0; comp <= KW; ++comp) {
        uint32_t* dst = (comp == 0 ? vout : kout + (comp - 1) * LN) + seg;
#pragma unroll
        for (int i = 0; i < SP_ITEMS; ++i)
            if (dig[i] < 256) buf[pos[i]] = cur[i];
        if (comp < KW) load_comp(comp + 1, cur);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SP_ITEMS; ++k) {
            const int sp = tid + k * NT;
            if (sp < nvalid) dst[doff[k]] = buf[sp];
        }
        __syncthreads();
    }
}

// ---- Top-word-first ordering ----
// The digit passes can run over the key's top word alone (its leading
// columns), moving that word and the ids. The lower words of every sorted
// position are then gathered from the packed keys in point order, and each run
// of equal top words is ordered by (lower words, id): the LSD passes leave a
// run's ids ascending, so this is the order the full sort produces.

// skeys[w][i] = keys0[w][table + ids[i]] for the lower words w < KW - 1; the
// sorted top words are copied into skeys' top slot unless they are there.
__global__ void k_gather_lower(const uint32_t* __restrict__ keys0, const uint32_t* __restrict__ ids,
                               const uint32_t* top, int64_t N, int L, int KW, uint32_t* skeys) {
    const int64_t LN = (int64_t)L * N, seg = (int64_t)blockIdx.y * N;
    uint32_t* stop = skeys + (int64_t)(KW - 1) * LN;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t idx = seg + i;
        const uint32_t id = ids[idx];
        for (int w = 0; w < KW - 1; ++w) skeys[w * LN + idx] = __ldg(keys0 + w * LN + seg + id);
        if (top != stop) stop[idx] = top[idx];
    }
}

// Runs of two or more equal top words, found from their first element, go to
// three lists by length: 2..8 (tiny), 9..32 (small), 33..kRunMax (large); a
// longer run or a full list sets cnt[3] (the caller then sorts all words
// instead). Block (x, table y); each thread examines RUN_ITEMS consecutive
// positions. List slots are claimed per block (shared counters, then one
// global atomic per block and class): with tens of thousands of runs per
// table, one global atomic per run or per warp serialises on the counters.
constexpr int RUN_ITEMS = 8;
__global__ void __launch_bounds__(NT) k_run_find(const uint32_t* __restrict__ top, int64_t N, RunLists rl) {
    __shared__ unsigned int sc[3], sbase[3];
    if (threadIdx.x < 3) sc[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t* t = top + (int64_t)blockIdx.y * N;
    const int64_t i0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * RUN_ITEMS;
    uint32_t len[RUN_ITEMS];
    unsigned int mine[3] = {0u, 0u, 0u};
#pragma unroll
    for (int k = 0; k < RUN_ITEMS; ++k) {
        const int64_t i = i0 + k;
        len[k] = 0;
        if (i + 1 < N) {
            const uint32_t v = t[i];
            if (t[i + 1] == v && !(i > 0 && t[i - 1] == v)) {
                int64_t j = i + 2;
                while (j < N && j - i <= kRunMax && t[j] == v) ++j;
                if (j - i > kRunMax) atomicOr(rl.cnt + 3, 1u);
                else len[k] = (uint32_t)(j - i);
            }
        }
        const uint32_t n = len[k];
        mine[0] += (n >= 2 && n <= 8) ? 1u : 0u;
        mine[1] += (n > 8 && n <= 32) ? 1u : 0u;
        mine[2] += n > 32 ? 1u : 0u;
    }
    unsigned int off[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) off[c] = mine[c] ? atomicAdd(&sc[c], mine[c]) : 0u;
    __syncthreads();
    if (threadIdx.x < 3) sbase[threadIdx.x] = sc[threadIdx.x] ? atomicAdd(rl.cnt + threadIdx.x, sc[threadIdx.x]) : 0u;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < RUN_ITEMS; ++k) {
        const uint32_t n = len[k];
        if (n < 2) continue;
        const int c = n <= 8 ? 0 : (n <= 32 ? 1 : 2);
        const unsigned int slot = sbase[c] + off[c]++;
        const unsigned int cap = c == 0 ? rl.tcap : (c == 1 ? rl.scap : rl.lcap);
        unsigned long long* pos = c == 0 ? rl.tpos : (c == 1 ? rl.spos : rl.lpos);
        uint32_t* lens = c == 0 ? rl.tlen : (c == 1 ? rl.slen : rl.llen);
        if (slot < cap) {
            pos[slot] = (unsigned long long)((int64_t)blockIdx.y * N + i0 + k);
            lens[slot] = n;
        } else {
            atomicOr(rl.cnt + 3, 2u);
        }
    }
}

// (lower words from the most significant down, then id) of a < of b
template <int KWL>
__device__ __forceinline__ bool run_less(const uint32_t (&a)[KWL + 1], const uint32_t (&b)[KWL + 1]) {
#pragma unroll
    for (int k = KWL - 1; k >= 0; --k)
        if (a[k] != b[k]) return a[k] < b[k];
    return a[KWL] < b[KWL];
}

// One thread per run of 2 to 8: an odd-even transposition sort over eight
// register slots (missing slots hold all-ones, above every element).
template <int KWL>
__global__ void k_run_sort_tiny(const unsigned long long* __restrict__ tpos, const uint32_t* __restrict__ tlen,
                                const unsigned int* __restrict__ cnt, unsigned int tcap, int64_t LN,
                                uint32_t* __restrict__ skeys, uint32_t* __restrict__ ids) {
    const unsigned int nrun = min(cnt[0], tcap);
    for (unsigned int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrun; r += gridDim.x * blockDim.x) {
        const int64_t pos = (int64_t)tpos[r];
        const int len = (int)tlen[r];
        uint32_t e[8][KWL + 1];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
#pragma unroll
            for (int k = 0; k <= KWL; ++k) e[t][k] = 0xFFFFFFFFu;
            if (t < len) {
#pragma unroll
                for (int k = 0; k < KWL; ++k) e[t][k] = skeys[k * LN + pos + t];
                e[t][KWL] = ids[pos + t];
            }
        }
#pragma unroll
        for (int ph = 0; ph < 8; ++ph) {
#pragma unroll
            for (int t = ph & 1; t + 1 < 8; t += 2) {
                if (run_less<KWL>(e[t + 1], e[t])) {
#pragma unroll
                    for (int k = 0; k <= KWL; ++k) {
                        const uint32_t x = e[t][k];
                        e[t][k] = e[t + 1][k];
                        e[t + 1][k] = x;
                    }
                }
            }
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            if (t < len) {
#pragma unroll
                for (int k = 0; k < KWL; ++k) skeys[k * LN + pos + t] = e[t][k];
                ids[pos + t] = e[t][KWL];
            }
        }
    }
}

// One warp per run of at most 32: a bitonic sort across the lanes (missing
// lanes hold all-ones, above every element: ids are below 2^32 - 1).
template <int KWL>
__global__ void k_run_sort_small(const unsigned long long* __restrict__ spos, const uint32_t* __restrict__ slen,
                                 const unsigned int* __restrict__ cnt, unsigned int scap, int64_t LN,
                                 uint32_t* __restrict__ skeys, uint32_t* __restrict__ ids) {
    const int lane = threadIdx.x & 31;
    const unsigned int nrun = min(cnt[1], scap);
    for (unsigned int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < nrun;
         r += (gridDim.x * blockDim.x) >> 5) {
        const int64_t pos = (int64_t)spos[r];
        const int len = (int)slen[r];
        uint32_t e[KWL + 1];
#pragma unroll
        for (int k = 0; k <= KWL; ++k) e[k] = 0xFFFFFFFFu;
        if (lane < len) {
#pragma unroll
            for (int k = 0; k < KWL; ++k) e[k] = skeys[k * LN + pos + lane];
            e[KWL] = ids[pos + lane];
        }
#pragma unroll
        for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
            for (int j = k >> 1; j > 0; j >>= 1) {
                uint32_t o[KWL + 1];
#pragma unroll
                for (int c = 0; c <= KWL; ++c) o[c] = __shfl_xor_sync(0xffffffffu, e[c], j);
                const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
                const bool o_less = run_less<KWL>(o, e);
                if (o_less == keep_min) {
#pragma unroll
                    for (int c = 0; c <= KWL; ++c) e[c] = o[c];
                }
            }
        }
        if (lane < len) {
#pragma unroll
            for (int k = 0; k < KWL; ++k) skeys[k * LN + pos + lane] = e[k];
            ids[pos + lane] = e[KWL];
        }
    }
}

// One block per run of 33 to kRunMax elements: a bitonic sort in shared memory.
template <int KWL>
__global__ void __launch_bounds__(NT) k_run_sort_large(const unsigned long long* __restrict__ lpos,
                                                      const uint32_t* __restrict__ llen,
                                                      const unsigned int* __restrict__ cnt, unsigned int lcap,
                                                      int64_t LN, uint32_t* __restrict__ skeys,
                                                      uint32_t* __restrict__ ids) {
    __shared__ uint32_t sv[KWL + 1][kRunMax];
    const unsigned int nrun = min(cnt[2], lcap);
    for (unsigned int r = blockIdx.x; r < nrun; r += gridDim.x) {
        const int64_t pos = (int64_t)lpos[r];
        const int len = (int)llen[r];
        int n2 = 64;
        while (n2 < len) n2 <<= 1;
        for (int t = threadIdx.x; t < n2; t += NT) {
#pragma unroll
            for (int k = 0; k < KWL; ++k) sv[k][t] = t < len ? skeys[k * LN + pos + t] : 0xFFFFFFFFu;
            sv[KWL][t] = t < len ? ids[pos + t] : 0xFFFFFFFFu;
        }
        __syncthreads();
        for (int k = 2; k <= n2; k <<= 1) {
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int t = threadIdx.x; t < n2; t += NT) {
                    const int u = t ^ j;
                    if (u > t) {
                        uint32_t a[KWL + 1], b[KWL + 1];
#pragma unroll
                        for (int c = 0; c <= KWL; ++c) {
                            a[c] = sv[c][t];
                            b[c] = sv[c][u];
                        }
                        const bool asc = (t & k) == 0;
                        if (run_less<KWL>(b, a) == asc) {
#pragma unroll
                            for (int c = 0; c <= KWL; ++c) {
                                sv[c][t] = b[c];
                                sv[c][u] = a[c];
                            }
                        }
                    }
                }
                __syncthreads();
            }
        }
        for (int t = threadIdx.x; t < len; t += NT) {
#pragma unroll
            for (int k = 0; k < KWL; ++k) skeys[k * LN + pos + t] = sv[k][t];
            ids[pos + t] = sv[KWL][t];
        }
        __syncthreads();
    }
}

__device__ __forceinline__ bool key_differs(const uint32_t* keys, int64_t LN, int64_t a, int64_t b, int KW) {
    for (int w = 0; w < KW; ++w)
        if (keys[w * LN + a] != keys[w * LN + b]) return true;
    return false;
}

__global__ void k_rl_count(const uint32_t* __restrict__ keys, int64_t N, int L, int KW, uint32_t* __restrict__ tile_cnt) {
    __shared__ uint32_t ws[SP_WARPS];
    const int l = blockIdx.y, tile = blockIdx.x, tiles = gridDim.x;
    const int64_t LN = (int64_t)L * N, seg = (int64_t)l * N;
    uint32_t c = 0;
    for (int e = threadIdx.x; e < SP_TILE; e += NT) {
        const int64_t i = (int64_t)tile * SP_TILE + e;
        if (i < N) c += (i == 0 || key_differs(keys, LN, seg + i, seg + i - 1, KW)) ? 1u : 0u;
    }
    uint32_t tot;
    block_excl_scan(c, ws, &tot);
    if (threadIdx.x == 0) tile_cnt[(int64_t)l * tiles + tile] = tot;
}

__global__ void k_rl_scan(const uint32_t* __restrict__ tile_cnt, int tiles, uint32_t* __restrict__ tile_off,
                          uint32_t* __restrict__ nb) {
    __shared__ uint32_t ws[SP_WARPS];
    const int l = blockIdx.x;
    uint32_t carry = 0;
    for (int t0 = 0; t0 < tiles; t0 += NT) {
        const int t = t0 + threadIdx.x;
        const uint32_t v = t < tiles ? tile_cnt[(int64_t)l * tiles + t] : 0;
        uint32_t tot;
        const uint32_t ex = block_excl_scan(v, ws, &tot);
        if (t < tiles) tile_off[(int64_t)l * tiles + t] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) nb[l] = carry;
}

// Bucket starts and unique keys of one tile of 4,096 sorted positions: warp w
// takes positions [512 w, 512 w + 512) as 16 rows of 32 lanes (coalesced key
// loads), ranks its flagged positions with ballots, and the block scans the
// warp totals; flagged positions are written in order.
__global__ void k_rl_write(const uint32_t* __restrict__ keys, int64_t N, int L, int KW,
                           const uint32_t* __restrict__ tile_off, const uint64_t* __restrict__ boff,
                           uint32_t* __restrict__ starts, uint32_t* __restrict__ ukeys) {
    __shared__ uint32_t ws[SP_WARPS];
    const int l = blockIdx.y, tile = blockIdx.x, tiles = gridDim.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t LN = (int64_t)L * N, seg = (int64_t)l * N;
    const int64_t w0 = (int64_t)tile * SP_TILE + (int64_t)warp * (32 * SP_ITEMS);
    uint32_t ball[SP_ITEMS];
    uint32_t c = 0;
#pragma unroll
    for (int k = 0; k < SP_ITEMS; ++k) {
        const int64_t i = w0 + k * 32 + lane;
        const bool f = i < N && (i == 0 || key_differs(keys, LN, seg + i, seg + i - 1, KW));
        ball[k] = __ballot_sync(0xffffffffu, f);
        c += __popc(ball[k]);
    }
    if (lane == 0) ws[warp] = c;
    __syncthreads();
    uint32_t r = tile_off[(int64_t)l * tiles + tile];
    for (int w = 0; w < warp; ++w) r += ws[w];
    const uint64_t bo = boff[l];
    const uint32_t below = (1u << lane) - 1u;
#pragma unroll
    for (int k = 0; k < SP_ITEMS; ++k) {
        if ((ball[k] >> lane) & 1u) {
            const int64_t i = w0 + k * 32 + lane;
            const uint64_t g = bo + r + __popc(ball[k] & below);
            starts[g] = (uint32_t)i;
            for (int w = 0; w < KW; ++w) ukeys[g * KW + w] = keys[w * LN + seg + i];
        }
        r += __popc(ball[k]);
    }
}

__global__ void k_bucket_sizes(const uint64_t* __restrict__ boff, const uint32_t* __restrict__ starts, int64_t N,
                               uint32_t* __restrict__ sizes, uint32_t* __restrict__ max_size) {
    const int l = blockIdx.y;
    const int64_t j = (int64_t)blockIdx.x * NT + threadIdx.x;
    const int64_t B = (int64_t)(boff[l + 1] - boff[l]);
    uint32_t sz = 0;
    if (j < B) {
        const uint64_t g = boff[l] + j;
        const int64_t end = (j + 1 < B) ? (int64_t)starts[g + 1] : N;
        sz = (uint32_t)(end - (int64_t)starts[g]);
        sizes[g] = sz;
    }
    // largest bucket: one atomic per block (one per warp serialises on the
    // single address when every bucket is small and there are millions)
    __shared__ uint32_t smax[SP_WARPS];
    const uint32_t wmax = __reduce_max_sync(0xffffffffu, sz);
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = wmax;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t m = 0;
        for (int w = 0; w < SP_WARPS; ++w) m = max(m, smax[w]);
        if (m) atomicMax(max_size, m);
    }
}

__global__ void k_hash_build(const uint64_t* __restrict__ boff, const uint32_t* __restrict__ ukeys, int M, int KW,
                             const uint16_t* __restrict__ foff, const uint8_t* __restrict__ fbits,
                             const unsigned long long* __restrict__ rmul, const uint64_t* __restrict__ hoff,
                             const uint32_t* __restrict__ hmask, unsigned long long* __restrict__ hslots,
                             uint32_t* __restrict__ filt, const uint64_t* __restrict__ fl_off,
                             const uint32_t* __restrict__ fl_mask, int* err) {
    const int l = blockIdx.y;
    const int64_t j = (int64_t)blockIdx.x * NT + threadIdx.x;
    const int64_t B = (int64_t)(boff[l + 1] - boff[l]);
    if (j >= B) return;
    const uint32_t* key = ukeys + (boff[l] + j) * KW;
    unsigned __int128 kk = 0;
    for (int w = KW - 1; w >= 0; --w) kk = (kk << 32) | key[w];
    const uint32_t gmask = hmask[l];
    uint64_t hs = 0;   // additive lookup hash over the key's fields
    // fields are contiguous from bit 0 (column M - 1) upwards
    for (int m = M - 1; m >= 0; --m) {
        const int c = l * M + m;
        const int bits = __ldg(fbits + c);
        const uint32_t f = bits ? (uint32_t)kk & (bits == 32 ? 0xFFFFFFFFu : ((1u << bits) - 1u)) : 0u;
        kk >>= bits;
        hs += (uint64_t)f * __ldg(rmul + c);
    }
    const uint64_t hh = hash_finish(hs);
    const uint32_t h = (uint32_t)hh;
    const uint32_t fp = slot_fp(hh);
    if (filt) {
        const uint32_t fx = filter_mix(hh);
        atomicOr(filt + fl_off[l] + (fx & fl_mask[l]), filter_bits(fx));
    }
    unsigned long long* slots = hslots + hoff[l];
    // Claim the first empty slot in probe order (a group's slots in order,
    // then the next group), then store the bucket index beside it. Lookups
    // stop at the first empty slot they meet, which can only lie past every
    // key inserted along the same path.
    for (uint32_t p = 0; p <= gmask; ++p) {
        unsigned long long* grp = slots + (uint64_t)((h + p) & gmask) * kGroupWords;
        unsigned long long cur = *reinterpret_cast<volatile unsigned long long*>(grp);
        // One 64-bit CAS per attempt on the group's fingerprint word; each
        // failure means another insert took a slot, so at most four tries.
        for (int tries = 0; tries <= kGroupSlots; ++tries) {
            int e = 0;
            while (e < kGroupSlots && ((cur >> (16 * e)) & 0xFFFFu) != kEmptyFp) ++e;
            if (e == kGroupSlots) break;   // group full: next group
            const unsigned long long nw = (cur & ~(0xFFFFull << (16 * e))) | ((unsigned long long)fp << (16 * e));
            const unsigned long long old = atomicCAS(grp, cur, nw);
            if (old == cur) {
                reinterpret_cast<uint32_t*>(grp + 1)[e] = (uint32_t)j;
                return;
            }
            cur = old;
        }
    }
    atomicOr(err, kErrHashFull);
}

__global__ void k_decode_codes(const uint64_t* __restrict__ boff, const uint32_t* __restrict__ ukeys, int M, int KW,
                               const int32_t* __restrict__ cmin, const uint8_t* __restrict__ fbits,
                               const uint16_t* __restrict__ foff, float* __restrict__ codes) {
    const int l = blockIdx.y;
    const int64_t j = (int64_t)blockIdx.x * NT + threadIdx.x;
    const int64_t B = (int64_t)(boff[l + 1] - boff[l]);
    if (j >= B) return;
    uint32_t k[kMaxKW];
    for (int w = 0; w < KW; ++w) k[w] = ukeys[(boff[l] + j) * KW + w];
    float* out = codes + boff[l] * M;
    for (int m = 0; m < M; ++m) {
        const int c = l * M + m;
        out[(int64_t)m * B + j] = (float)(int32_t)(key_get(k, foff[c], fbits[c]) + (uint32_t)cmin[c]);
    }
}

__global__ void k_codes_minmax(const uint64_t* __restrict__ boff, const float* __restrict__ codes, int M,
                               int32_t* __restrict__ cmin, int32_t* __restrict__ cmax, int* err) {
    __shared__ int32_t slo[SP_WARPS], shi[SP_WARPS];
    const int l = blockIdx.y;
    const int64_t j = (int64_t)blockIdx.x * NT + threadIdx.x;
    const int64_t B = (int64_t)(boff[l + 1] - boff[l]);
    if ((int64_t)blockIdx.x * NT >= B) return;  // whole block idle: uniform exit
    const float* in = codes + boff[l] * M;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int m = 0; m < M; ++m) {
        int32_t lo = INT_MAX, hi = INT_MIN;
        if (j < B) {
            const float f = in[(int64_t)m * B + j];
            if (!(f == floorf(f) && f >= -2147483648.0f && f < 2147483648.0f)) {
                atomicOr(err, kErrNotIntegral);
            } else {
                lo = hi = (int32_t)f;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) {
            slo[w] = lo;
            shi[w] = hi;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int k = 1; k < SP_WARPS; ++k) {
                lo = min(lo, slo[k]);
                hi = max(hi, shi[k]);
            }
            atomicMin(&cmin[l * M + m], lo);
            atomicMax(&cmax[l * M + m], hi);
        }
        __syncthreads();
    }
}

__global__ void k_pack_from_codes(const uint64_t* __restrict__ boff, const float* __restrict__ codes, int M, int KW,
                                  const int32_t* __restrict__ cmin, const uint8_t* __restrict__ fbits,
                                  const uint16_t* __restrict__ foff, uint32_t* __restrict__ ukeys) {
    const int l = blockIdx.y;
    const int64_t j = (int64_t)blockIdx.x * NT + threadIdx.x;
    const int64_t B = (int64_t)(boff[l + 1] - boff[l]);
    if (j >= B) return;
    const float* in = codes + boff[l] * M;
    uint32_t k[kMaxKW];
#pragma unroll
    for (int w = 0; w < kMaxKW; ++w) k[w] = 0;
    for (int m = 0; m < M; ++m) {
        const int c = l * M + m;
        if (fbits[c]) key_put(k, foff[c], fbits[c], (uint32_t)((int32_t)in[(int64_t)m * B + j] - cmin[c]));
    }
    for (int w = 0; w < KW; ++w) ukeys[(boff[l] + j) * KW + w] = k[w];
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC 2011), keyed by the seed, counter = element index.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

__global__ void k_random(float* __restrict__ A, float* __restrict__ u, int64_t nA, int64_t nu,
                         unsigned long long seed) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
    if (i < nA) {
        const uint4 r = philox4x32_10(make_uint4((uint32_t)i, (uint32_t)(i >> 32), 0u, 0u), key);
        const float u1 = ((r.x >> 8) + 1u) * (1.0f / 16777216.0f);   // (0, 1]
        const float u2 = (r.y >> 8) * (1.0f / 16777216.0f);          // [0, 1)
        A[i] = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);          // Box-Muller
    }
    if (i < nu) {
        const uint4 r = philox4x32_10(make_uint4((uint32_t)i, (uint32_t)(i >> 32), 1u, 0u), key);
        u[i] = ((r.x >> 8) + 1u) * (1.0f / 16777216.0f);
    }
}

inline int blocks_for(int64_t n) { return (int)((n + NT - 1) / NT); }

}  // namespace

cudaError_t launch_pack_keys(const int32_t* codes, int64_t N, int L, int M, int KW, const int32_t* cmin,
                             const uint8_t* fbits, const uint16_t* foff, uint32_t* keys, uint32_t* vals,
                             cudaStream_t st) {
    const int64_t LN = (int64_t)L * N;
    const int grid = (int)std::min<int64_t>((LN + NT - 1) / NT, 152 * 32);
    k_pack_keys<<<grid, NT, 0, st>>>(codes, N, L, M, KW, cmin, fbits, foff, keys, vals);
    return cudaGetLastError();
}

size_t sort_status_words(int64_t N, int L) {
    const int64_t tiles = (N + SP_TILE - 1) / SP_TILE;
    return (size_t)(L * tiles * 256 + 32);
}

cudaError_t run_segmented_sort(SortBuffers& sb, int64_t N, int L, int KW, int passes, bool* result_in_alt,
                               cudaStream_t st) {
    *result_in_alt = false;
    if (passes <= 0 || N <= 1) return cudaSuccess;
    const int tiles = (int)((N + SP_TILE - 1) / SP_TILE);
    cudaError_t e;
    if ((e = cudaMemsetAsync(sb.hist, 0, sizeof(uint32_t) * L * passes * 256, st)) != cudaSuccess) return e;
    const dim3 hg((unsigned)((N + HIST_CHUNK - 1) / HIST_CHUNK), L);
    k_sort_hist<<<hg, NT, passes * 256 * sizeof(uint32_t), st>>>(sb.keys[0], N, L, passes, sb.hist);
    k_sort_digit_base<<<L * passes, NT, 0, st>>>(sb.hist, sb.base);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // Skip digit passes that are constant over every table (a stable pass
    // with one occupied bin is the identity).
    const size_t hwords = (size_t)L * passes * 256, hbytes = sizeof(uint32_t) * hwords;
    const bool own = sb.h_hist == nullptr || sb.h_hist_words < hwords;
    uint32_t* h_hist = own ? nullptr : sb.h_hist;
    if (own && (e = cudaMallocHost(&h_hist, hbytes)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(h_hist, sb.hist, hbytes, cudaMemcpyDeviceToHost, st)) == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        if (own) cudaFreeHost(h_hist);
        return e;
    }
    int cur = 0;
    const size_t status_words = sort_status_words(N, L);
    uint32_t* counter = sb.status + (status_words - 32);
    for (int p = 0; p < passes; ++p) {
        bool trivial = true;
        for (int l = 0; l < L && trivial; ++l) {
            const uint32_t* hp = h_hist + ((size_t)l * passes + p) * 256;
            int nz = 0;
            for (int d = 0; d < 256; ++d) nz += hp[d] != 0;
            trivial = nz <= 1;
        }
        if (trivial) continue;
        if ((e = cudaMemsetAsync(sb.status, 0, sizeof(uint32_t) * status_words, st)) != cudaSuccess) break;
        k_sort_pass<<<(unsigned)(L * tiles), NT, 0, st>>>(sb.keys[cur], sb.vals[cur], sb.keys[cur ^ 1],
                                                          sb.vals[cur ^ 1], N, L, KW, tiles, p >> 2, (p & 3) * 8,
                                                          sb.base, passes, p, sb.status, counter, sb.err);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        cur ^= 1;
    }
    if (own) cudaFreeHost(h_hist);
    *result_in_alt = cur == 1;
    return e;
}

cudaError_t launch_gather_lower(const uint32_t* keys0, const uint32_t* ids, const uint32_t* top, int64_t N, int L,
                                int KW, uint32_t* skeys, cudaStream_t st) {
    const dim3 grid((unsigned)std::min<int64_t>((N + NT - 1) / NT, 152 * 4), (unsigned)L);
    k_gather_lower<<<grid, NT, 0, st>>>(keys0, ids, top, N, L, KW, skeys);
    return cudaGetLastError();
}

cudaError_t launch_run_find(const uint32_t* top, int64_t N, int L, const RunLists& rl, cudaStream_t st) {
    const int64_t LN = (int64_t)L * N;
    cudaError_t e = cudaMemsetAsync(rl.cnt, 0, 4 * sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    (void)LN;
    const dim3 grid((unsigned)((N + (int64_t)NT * RUN_ITEMS - 1) / ((int64_t)NT * RUN_ITEMS)), (unsigned)L);
    k_run_find<<<grid, NT, 0, st>>>(top, N, rl);
    return cudaGetLastError();
}

int run_max_len() { return kRunMax; }

template <int KWL>
void launch_run_sorts_w(const RunLists& rl, unsigned int ntiny, unsigned int nsmall, unsigned int nlarge, int64_t LN,
                        uint32_t* skeys, uint32_t* ids, cudaStream_t st) {
    const unsigned gt = (unsigned)std::min<unsigned long long>(((unsigned long long)ntiny + NT - 1) / NT, 152 * 16);
    const unsigned gs = (unsigned)std::min<unsigned long long>(((unsigned long long)nsmall * 32 + NT - 1) / NT, 152 * 32);
    const unsigned gl = (unsigned)std::min<unsigned int>(nlarge, 152 * 4);
    if (gt) k_run_sort_tiny<KWL><<<gt, NT, 0, st>>>(rl.tpos, rl.tlen, rl.cnt, rl.tcap, LN, skeys, ids);
    if (gs) k_run_sort_small<KWL><<<gs, NT, 0, st>>>(rl.spos, rl.slen, rl.cnt, rl.scap, LN, skeys, ids);
    if (gl) k_run_sort_large<KWL><<<gl, NT, 0, st>>>(rl.lpos, rl.llen, rl.cnt, rl.lcap, LN, skeys, ids);
}

cudaError_t launch_run_sorts(const RunLists& rl, const unsigned int* counts, int64_t N, int L, int KW, uint32_t* skeys,
                             uint32_t* ids, cudaStream_t st) {
    const int64_t LN = (int64_t)L * N;
    switch (KW - 1) {
    case 1: launch_run_sorts_w<1>(rl, counts[0], counts[1], counts[2], LN, skeys, ids, st); break;
    case 2: launch_run_sorts_w<2>(rl, counts[0], counts[1], counts[2], LN, skeys, ids, st); break;
    case 3: launch_run_sorts_w<3>(rl, counts[0], counts[1], counts[2], LN, skeys, ids, st); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_rl_count(const uint32_t* keys, int64_t N, int L, int KW, uint32_t* tile_cnt, uint32_t* tile_off,
                            uint32_t* nb, cudaStream_t st) {
    const int tiles = (int)((N + SP_TILE - 1) / SP_TILE);
    k_rl_count<<<dim3(tiles, L), NT, 0, st>>>(keys, N, L, KW, tile_cnt);
    k_rl_scan<<<L, NT, 0, st>>>(tile_cnt, tiles, tile_off, nb);
    return cudaGetLastError();
}

cudaError_t launch_rl_write(const uint32_t* keys, int64_t N, int L, int KW, const uint32_t* tile_off,
                            const uint64_t* boff, uint32_t* starts, uint32_t* ukeys, cudaStream_t st) {
    const int tiles = (int)((N + SP_TILE - 1) / SP_TILE);
    k_rl_write<<<dim3(tiles, L), NT, 0, st>>>(keys, N, L, KW, tile_off, boff, starts, ukeys);
    return cudaGetLastError();
}

cudaError_t launch_bucket_sizes(const uint64_t* boff, const uint32_t* starts, int64_t N, int L, int64_t maxB,
                                uint32_t* sizes, uint32_t* max_size, cudaStream_t st) {
    if (maxB <= 0) return cudaSuccess;
    k_bucket_sizes<<<dim3(blocks_for(maxB), L), NT, 0, st>>>(boff, starts, N, sizes, max_size);
    return cudaGetLastError();
}

cudaError_t launch_hash_build(const uint64_t* boff, const uint32_t* ukeys, int L, int M, int KW, int64_t maxB,
                              const uint16_t* foff, const uint8_t* fbits, const unsigned long long* rmul,
                              const uint64_t* hoff, const uint32_t* hmask, unsigned long long* hslots,
                              uint32_t* filt, const uint64_t* fl_off, const uint32_t* fl_mask, int* err,
                              cudaStream_t st) {
    if (maxB <= 0) return cudaSuccess;
    k_hash_build<<<dim3(blocks_for(maxB), L), NT, 0, st>>>(boff, ukeys, M, KW, foff, fbits, rmul, hoff, hmask,
                                                          hslots, filt, fl_off, fl_mask, err);
    return cudaGetLastError();
}

cudaError_t launch_decode_codes(const uint64_t* boff, const uint32_t* ukeys, int L, int M, int KW, int64_t maxB,
                                const int32_t* cmin, const uint8_t* fbits, const uint16_t* foff, float* codes,
                                cudaStream_t st) {
    if (maxB <= 0) return cudaSuccess;
    k_decode_codes<<<dim3(blocks_for(maxB), L), NT, 0, st>>>(boff, ukeys, M, KW, cmin, fbits, foff, codes);
    return cudaGetLastError();
}

cudaError_t launch_codes_minmax(const uint64_t* boff, const float* codes, int L, int M, int64_t maxB,
                                int32_t* cmin, int32_t* cmax, int* err, cudaStream_t st) {
    if (maxB <= 0) return cudaSuccess;
    k_codes_minmax<<<dim3(blocks_for(maxB), L), NT, 0, st>>>(boff, codes, M, cmin, cmax, err);
    return cudaGetLastError();
}

cudaError_t launch_pack_from_codes(const uint64_t* boff, const float* codes, int L, int M, int KW, int64_t maxB,
                                   const int32_t* cmin, const uint8_t* fbits, const uint16_t* foff, uint32_t* ukeys,
                                   cudaStream_t st) {
    if (maxB <= 0) return cudaSuccess;
    k_pack_from_codes<<<dim3(blocks_for(maxB), L), NT, 0, st>>>(boff, codes, M, KW, cmin, fbits, foff, ukeys);
    return cudaGetLastError();
}

cudaError_t launch_random_projection(float* A, float* u, int64_t nA, int64_t nu, unsigned long long seed,
                                     cudaStream_t st) {
    const int64_t n = std::max(nA, nu);
    if (n <= 0) return cudaSuccess;
    k_random<<<blocks_for(n), NT, 0, st>>>(A, u, nA, nu, seed);
    return cudaGetLastError();
}

}  // namespace culsh
