// K4: the query path.
//
// k_probe (one thread per (table, query)) replaces cuLSH_Kernels.cu:266-289
// (kernel_calculateDeltas), cuLSH_Kernels.cu:144-257 (balanceHeap_deltas +
// kernel_calculateProbingCodes), cuLSH_Querying.cu:63-119 (the host round trip
// that scatters home codes) and the whole sort-merge bucket match of
// cuLSH_Querying.cu:124-165 + cuLSH_Kernels.cu:124-138: every probe code is
// packed into the table's key layout and looked up in the open-addressing hash
// built at index time, verified against the stored bucket key. It also sums
// the non-unique candidate counts of cuLSH_SearchTables.cu:250-255.
//
// k_candidates (one 128-thread block per query) replaces the host collect /
// sort / unique of cuLSH_SearchTables.cu:321-364, the per-query fill_n of
// :384-389, kernel_calculateDistances (cuLSH_Kernels.cu:301-348) and the top-K
// kernels (cuLSH_Kernels.cu:356-456): bucket ids are gathered straight from the
// sorted id arrays, deduplicated in a shared-memory hash set (global arena for
// large sets), squared L2 distances are computed in the reference's lane order
// from 16-byte loads, and each warp keeps a sorted top-K that the block merges.
#include <cfloat>

#include "culsh_internal.cuh"

namespace culsh {
namespace {

constexpr int CT = 128;
constexpr int CW = CT / 32;
constexpr int SM_SLOTS = 4096;
constexpr int SM_CAP = SM_SLOTS / 2;
constexpr uint32_t kEmpty32 = 0xFFFFFFFFu;

__device__ __forceinline__ int ceil_log2_dev(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

// Max-heap sift-down over delta indices; an empty slot (-1) ranks above every
// delta (cuLSH_Kernels.cu:144-175).
__device__ void sift_deltas(int8_t* perm, const float* dl, int total, int levels) {
    int parent = 0;
    for (int level = 0; level < levels - 1; ++level) {
        const int left = parent * 2 + 1, right = left + 1;
        int mx = parent;
        if (left < total && perm[left] == -1) {
            mx = left;
        } else if (right < total && perm[right] == -1) {
            mx = right;
        } else {
            if (left < total && dl[perm[left]] > dl[perm[mx]]) mx = left;
            if (right < total && dl[perm[right]] > dl[perm[mx]]) mx = right;
        }
        if (mx == parent) break;
        const int8_t t = perm[parent];
        perm[parent] = perm[mx];
        perm[mx] = t;
        parent = mx;
    }
}

// Exact-code lookup of one probe row in table l; returns the bucket index
// within the table or -1.
__device__ int32_t lookup_row(const LookupView& lv, int l, const float* row) {
    uint32_t key[kMaxKW];
#pragma unroll
    for (int w = 0; w < kMaxKW; ++w) key[w] = 0;
    const int M = lv.M, KW = lv.KW;
    for (int m = 0; m < M; ++m) {
        const int c = l * M + m;
        const float f = row[m];
        if (!(f >= -2147483648.0f && f < 2147483648.0f)) return -1;
        const int32_t ci = (int32_t)f;
        const int32_t lo = __ldg(lv.cmin + c);
        if (ci < lo || ci > __ldg(lv.cmax + c)) return -1;
        const int bits = __ldg(lv.fbits + c);
        if (bits) key_put(key, __ldg(lv.foff + c), bits, (uint32_t)(ci - lo));
    }
    const uint32_t mask = __ldg(lv.hmask + l);
    const uint32_t h = key_hash(key, KW, kSeedSlot);
    const uint32_t fp = key_hash(key, KW, kSeedFp);
    const unsigned long long* slots = lv.hslots + __ldg(lv.hoff + l);
    const uint64_t bo = __ldg(lv.boff + l);
    for (uint32_t p = 0; p <= mask; ++p) {
        const unsigned long long s = __ldg(slots + ((h + p) & mask));
        if (s == kEmptySlot) return -1;
        if ((uint32_t)(s >> 32) == fp) {
            const uint32_t j = (uint32_t)s;
            const uint32_t* uk = lv.ukeys + (bo + j) * KW;
            bool eq = true;
            for (int w = 0; w < KW; ++w) eq &= __ldg(uk + w) == key[w];
            if (eq) return (int32_t)j;
        }
    }
    return -1;
}

__global__ void __launch_bounds__(128) k_probe(ProbeArgs a) {
    const LookupView& lv = a.lv;
    const int Q = a.Q, T = a.T, L = lv.L, M = lv.M;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)L * Q) return;
    const int l = (int)(idx / Q), q = (int)(idx - (int64_t)l * Q);

    float home[kMaxM], row[kMaxM], dl[2 * kMaxM];
    for (int m = 0; m < M; ++m) {
        const float v = a.vals[(int64_t)(l * M + m) * Q + q];
        const float f = floorf(v);
        const float down = __fsub_rn(v, f);
        home[m] = f;
        dl[m] = down;
        dl[m + M] = __fsub_rn(1.0f, down);
    }
    int32_t* qb = a.qbuckets + (int64_t)l * Q * T + (int64_t)q * T;
    const uint64_t bo = lv.boff[l];
    unsigned long long cnu = 0;
    {
        const int32_t j = lookup_row(lv, l, home);
        qb[0] = j;
        if (j >= 0) cnu += lv.sizes[bo + j];
    }
    if (T > 1) {
        // Heap selection of the (at most 64) smallest deltas, then heap sort
        // into ascending order (cuLSH_Kernels.cu:202-214).
        const int maxT = min(2 * M, 64);
        const int levels = ceil_log2_dev(2 * M + 1);
        int8_t perm[64];
        for (int i = 0; i < maxT; ++i) perm[i] = -1;
        for (int i = 0; i < 2 * M; ++i) {
            if (perm[0] == -1 || dl[i] < dl[perm[0]]) {
                perm[0] = (int8_t)i;
                sift_deltas(perm, dl, maxT, levels);
            }
        }
        for (int i = maxT - 1; i > 0; --i) {
            const int8_t t = perm[0];
            perm[0] = perm[i];
            perm[i] = t;
            sift_deltas(perm, dl, i, levels);
        }
        // Shift / expand enumeration with a linear minimum search
        // (cuLSH_Kernels.cu:216-255); 64-bit masks.
        uint64_t comb[kMaxT];
        float cd[kMaxT];
        comb[0] = 1;
        cd[0] = dl[perm[0]];
        int size = 1;
        for (int t = 1; t < T; ++t) {
            float mn = FLT_MAX;
            int mi = 0;
            for (int i = 0; i < size; ++i) {
                if (cd[i] < mn) {
                    mi = i;
                    mn = cd[i];
                }
            }
            uint64_t probe = comb[mi];
            for (int m = 0; m < M; ++m) row[m] = home[m];
            int top = 0;
            for (uint64_t bitsleft = probe; bitsleft; bitsleft &= bitsleft - 1) {
                const int i = __ffsll((long long)bitsleft) - 1;
                const int pi = perm[i];
                const int m = pi % M;
                row[m] = __fadd_rn(row[m], pi >= M ? 1.0f : -1.0f);
                top = i;
            }
            if (top < maxT - 1) {
                probe |= 1ull << (top + 1);
                mn = __fadd_rn(mn, dl[perm[top + 1]]);
                comb[mi] = probe;
                cd[mi] = mn;
                probe -= 1ull << top;
                mn = __fsub_rn(mn, dl[perm[top]]);
                comb[size] = probe;
                cd[size] = mn;
                ++size;
            }
            const int32_t j = lookup_row(lv, l, row);
            qb[t] = j;
            if (j >= 0) cnu += lv.sizes[bo + j];
        }
    }
    if (cnu) atomicAdd(a.cnu + q, cnu);
}

__device__ __forceinline__ bool lessp(float a, uint32_t ai, float b, uint32_t bi) {
    return a < b || (a == b && ai < bi);
}

// Inserts (d, id) into a warp's sorted list [0, n) of capacity K; all lanes
// call it with the same arguments. Keeps ascending (distance, id) order.
__device__ __forceinline__ void warp_insert(float* wd, uint32_t* wi, int& n, int K, float d, uint32_t id,
                                            float& thr_d, uint32_t& thr_i) {
    const int lane = threadIdx.x & 31;
    int pos = 0;
    for (int b = 0; b < n; b += 32) {
        const int e = b + lane;
        const bool lt = e < n && lessp(wd[e], wi[e], d, id);
        pos += __popc(__ballot_sync(0xffffffffu, lt));
    }
    if (pos >= K) return;
    const int newn = min(n + 1, K);
    for (int hi = newn - 1; hi > pos; hi -= 32) {
        const int e = hi - lane;
        const bool act = e > pos;
        float vd = 0.f;
        uint32_t vi = 0;
        if (act) {
            vd = wd[e - 1];
            vi = wi[e - 1];
        }
        __syncwarp();
        if (act) {
            wd[e] = vd;
            wi[e] = vi;
        }
        __syncwarp();
    }
    if (lane == 0) {
        wd[pos] = d;
        wi[pos] = id;
    }
    __syncwarp();
    n = newn;
    if (n == K) {
        thr_d = wd[K - 1];
        thr_i = wi[K - 1];
    }
}

__device__ __forceinline__ void set_insert(uint32_t* hset, uint32_t mask, uint32_t* ulist, uint32_t* ucount,
                                           uint32_t id) {
    uint32_t h = mix32(id) & mask;
    for (uint32_t p = 0; p <= mask; ++p) {
        const uint32_t prev = atomicCAS(&hset[h], kEmpty32, id);
        if (prev == kEmpty32) {
            ulist[atomicAdd(ucount, 1u)] = id;
            return;
        }
        if (prev == id) return;
        h = (h + 1) & mask;
    }
}

__global__ void __launch_bounds__(CT) k_candidates(CandArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t s_ucount;
    __shared__ int s_ok;
    __shared__ unsigned long long s_off;
    __shared__ int s_wn[CW];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int q = a.qlist ? a.qlist[blockIdx.x] : (int)blockIdx.x;
    const int D = a.D, K = a.K, L = a.L, T = a.T;
    const int Dp = (D + 3) & ~3;
    float* qs = reinterpret_cast<float*>(smem);
    uint32_t* sh_set = reinterpret_cast<uint32_t*>(qs + Dp);
    uint32_t* sh_list = sh_set + SM_SLOTS;
    float* wd_all = reinterpret_cast<float*>(sh_list + SM_CAP);
    uint32_t* wi_all = reinterpret_cast<uint32_t*>(wd_all + CW * K);

    const unsigned long long C = a.cnu[q];
    int32_t* oid = a.out_ids + (int64_t)q * K;
    float* od = a.out_d + (int64_t)q * K;
    if (C == 0) {
        for (int k = tid; k < K; k += CT) {
            oid[k] = -1;
            od[k] = FLT_MAX;
        }
        if (tid == 0) a.cu[q] = 0;
        return;
    }

    uint32_t* hset = sh_set;
    uint32_t* ulist = sh_list;
    uint32_t cap = SM_SLOTS;
    if (C > (unsigned long long)SM_CAP) {
        unsigned long long c2 = 1;
        while (c2 < 2 * C) c2 <<= 1;
        if (tid == 0) {
            const unsigned long long need = c2 + C;
            const unsigned long long off = atomicAdd(a.arena_top, need);
            s_ok = off + need <= a.arena_words;
            s_off = off;
            if (!s_ok) a.deferred[atomicAdd(a.n_deferred, 1u)] = q;
        }
        __syncthreads();
        if (!s_ok) return;
        hset = a.arena + s_off;
        cap = (uint32_t)c2;
        ulist = hset + cap;
    }
    for (int i = tid; i < Dp; i += CT) qs[i] = i < D ? a.queries[(int64_t)q * D + i] : 0.0f;
    for (uint32_t i = tid; i < cap; i += CT) hset[i] = kEmpty32;
    if (tid == 0) s_ucount = 0;
    __syncthreads();

    // Gather every matched bucket's ids (duplicate probes included, as the
    // reference's candidate lists are) and deduplicate them.
    const int LT = L * T;
    const uint32_t mask = cap - 1;
    for (int e = warp; e < LT; e += CW) {
        const int l = e / T, t = e - l * T;
        const int32_t j = a.qbuckets[(int64_t)l * a.Q * T + (int64_t)q * T + t];
        if (j < 0) continue;
        const uint64_t g = a.boff[l] + (uint32_t)j;
        const uint32_t st = a.starts[g], sz = a.sizes[g];
        const uint32_t* src = a.ids + (int64_t)l * a.N + st;
        for (uint32_t k = lane; k < sz; k += 32) set_insert(hset, mask, ulist, &s_ucount, __ldg(src + k));
    }
    __syncthreads();
    const uint32_t U = s_ucount;

    // Distances in the reference lane order, per-warp sorted top-K.
    float* wd = wd_all + warp * K;
    uint32_t* wi = wi_all + warp * K;
    int n = 0;
    float thr_d = FLT_MAX;
    uint32_t thr_i = 0;
    const bool vec = (D & 3) == 0;
    const int per = vec ? 16 : 4;   // candidates per warp iteration
    for (uint32_t base = warp * per; base < U; base += CW * per) {
        float dist = 0.f;
        uint32_t id = 0;
        bool own;
        if (vec) {
            const uint32_t ci = base + (lane >> 1);
            const int h = lane & 1;
            const bool valid = ci < U;
            id = valid ? ulist[ci] : 0u;
            const float* rowp = a.X + (int64_t)id * D;
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
            if (valid) {
                for (int c = 4 * h; c < D; c += 8) {
                    const float4 x = __ldg(reinterpret_cast<const float4*>(rowp + c));
                    const float4 qv = *reinterpret_cast<const float4*>(qs + c);
                    const float d0 = __fsub_rn(qv.x, x.x), d1 = __fsub_rn(qv.y, x.y);
                    const float d2 = __fsub_rn(qv.z, x.z), d3 = __fsub_rn(qv.w, x.w);
                    s0 = __fmaf_rn(d0, d0, s0);
                    s1 = __fmaf_rn(d1, d1, s1);
                    s2 = __fmaf_rn(d2, d2, s2);
                    s3 = __fmaf_rn(d3, d3, s3);
                }
            }
            const float o0 = __shfl_xor_sync(0xffffffffu, s0, 1), o1 = __shfl_xor_sync(0xffffffffu, s1, 1);
            const float o2 = __shfl_xor_sync(0xffffffffu, s2, 1), o3 = __shfl_xor_sync(0xffffffffu, s3, 1);
            const float t0 = __fadd_rn(s0, o0), t1 = __fadd_rn(s1, o1), t2 = __fadd_rn(s2, o2), t3 = __fadd_rn(s3, o3);
            dist = __fadd_rn(__fadd_rn(t0, t2), __fadd_rn(t1, t3));
            own = valid && h == 0;
        } else {
            const uint32_t ci = base + (lane >> 3);
            const int r = lane & 7;
            const bool valid = ci < U;
            id = valid ? ulist[ci] : 0u;
            const float* rowp = a.X + (int64_t)id * D;
            float s = 0.f;
            if (valid)
                for (int c = r; c < D; c += 8) {
                    const float df = __fsub_rn(qs[c], __ldg(rowp + c));
                    s = __fmaf_rn(df, df, s);
                }
            const float t = __fadd_rn(s, __shfl_xor_sync(0xffffffffu, s, 4));
            const float u = __fadd_rn(t, __shfl_xor_sync(0xffffffffu, t, 2));
            dist = __fadd_rn(u, __shfl_xor_sync(0xffffffffu, u, 1));
            own = valid && r == 0;
        }
        uint32_t want = __ballot_sync(0xffffffffu, own && lessp(dist, id, thr_d, thr_i));
        while (want) {
            const int src = __ffs(want) - 1;
            want &= want - 1;
            const float cdv = __shfl_sync(0xffffffffu, dist, src);
            const uint32_t cid = __shfl_sync(0xffffffffu, id, src);
            if (lessp(cdv, cid, thr_d, thr_i)) warp_insert(wd, wi, n, K, cdv, cid, thr_d, thr_i);
        }
    }
    if (lane == 0) s_wn[warp] = n;
    __syncthreads();
    if (warp == 0) {
        for (int w = 1; w < CW; ++w) {
            const int nw = s_wn[w];
            const float* od2 = wd_all + w * K;
            const uint32_t* oi2 = wi_all + w * K;
            for (int e = 0; e < nw; ++e) {
                const float d = od2[e];
                const uint32_t id = oi2[e];
                if (!lessp(d, id, thr_d, thr_i)) break;
                warp_insert(wd, wi, n, K, d, id, thr_d, thr_i);
            }
        }
        for (int k = lane; k < K; k += 32) {
            oid[k] = k < n ? (int32_t)wi[k] : -1;
            od[k] = k < n ? wd[k] : FLT_MAX;
        }
        if (lane == 0) {
            a.cu[q] = U;
            atomicAdd(a.totals + 0, (unsigned long long)U);
            atomicAdd(a.totals + 1, C);
        }
    }
}

}  // namespace

cudaError_t launch_probe(const ProbeArgs& a, cudaStream_t st) {
    const int64_t n = (int64_t)a.lv.L * a.Q;
    if (n <= 0) return cudaSuccess;
    k_probe<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(a);
    return cudaGetLastError();
}

int cand_smem_capacity() { return SM_CAP; }

size_t cand_arena_words(unsigned long long nonunique) {
    if (nonunique <= (unsigned long long)SM_CAP) return 0;
    unsigned long long c2 = 1;
    while (c2 < 2 * nonunique) c2 <<= 1;
    return (size_t)(c2 + nonunique);
}

cudaError_t launch_candidates(const CandArgs& a, cudaStream_t st) {
    const int nblk = a.qlist ? a.nq : a.Q;
    if (nblk <= 0) return cudaSuccess;
    const size_t smem = sizeof(float) * (size_t)((a.D + 3) & ~3) + sizeof(uint32_t) * (SM_SLOTS + SM_CAP) +
                        (size_t)CW * a.K * (sizeof(float) + sizeof(uint32_t));
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(k_candidates, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    k_candidates<<<nblk, CT, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace culsh
