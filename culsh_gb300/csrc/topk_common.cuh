// Device helpers shared by the candidate kernels: the (distance, id) order of
// the top-K, a warp's sorted top-K list, and the open-addressing id set used
// to deduplicate candidates.
#pragma once

#include "culsh_internal.cuh"

namespace culsh {

constexpr uint32_t kEmpty32 = 0xFFFFFFFFu;

// Ascending (distance, id): ties go to the smaller id.
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

// Inserts id into the open-addressing set hset[0..mask]; a new id is appended
// to ulist when its position is below lcap. *ucount counts every new id, so a
// count above lcap reports an overflow without writing past the list.
__device__ __forceinline__ void set_insert(uint32_t* hset, uint32_t mask, uint32_t* ulist, uint32_t lcap,
                                           uint32_t* ucount, uint32_t id) {
    uint32_t h = mix32(id) & mask;
    for (uint32_t p = 0; p <= mask; ++p) {
        const uint32_t prev = atomicCAS(&hset[h], kEmpty32, id);
        if (prev == kEmpty32) {
            const uint32_t pos = atomicAdd(ucount, 1u);
            if (pos < lcap) ulist[pos] = id;
            return;
        }
        if (prev == id) return;
        h = (h + 1) & mask;
    }
}

// Exact FP32 squared distances, in the reference lane order
// (cuLSH_Kernels.cu:301-348), of list entries [0, cnt) into this warp's sorted
// top-K list (wd, wi, n, thr_d, thr_i). Entry j is candidate ci = idx_of(j)
// with point id id_at(ci); an entry whose exact distance is already known
// (pre(ci, d) returns true) is not loaded. With D % 4 == 0 two lanes share a
// candidate and each holds four of the eight lane partials from 16-byte
// loads; otherwise eight lanes share one. Every lane reaches every shuffle.
// All lanes of the warp call this with the same arguments.
template <int WW, class IdxOf, class IdAt, class Pre>
__device__ __forceinline__ void fp32_dist_pass(const float* __restrict__ X, int D, const float* qs, bool vec,
                                               uint32_t cnt, IdxOf idx_of, IdAt id_at, Pre pre, float* wd,
                                               uint32_t* wi, int K, int& n, float& thr_d, uint32_t& thr_i) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int per = vec ? 16 : 4;
    for (uint32_t base = warp * per; base < cnt; base += WW * per) {
        float dist = 0.f;
        uint32_t id = 0;
        bool own;
        if (vec) {
            const uint32_t j = base + (lane >> 1);
            const int h = lane & 1;
            const bool valid = j < cnt;
            const uint32_t ci = valid ? idx_of(j) : 0u;
            id = valid ? id_at(ci) : 0u;
            float pd = 0.f;
            const bool have = valid && pre(ci, pd);
            const float* rowp = X + (int64_t)id * D;
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
            if (valid && !have) {
#pragma unroll 8
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
            const float v = __fadd_rn(__fadd_rn(t0, t2), __fadd_rn(t1, t3));
            dist = have ? pd : v;
            own = valid && h == 0;
        } else {
            const uint32_t j = base + (lane >> 3);
            const int r = lane & 7;
            const bool valid = j < cnt;
            const uint32_t ci = valid ? idx_of(j) : 0u;
            id = valid ? id_at(ci) : 0u;
            float pd = 0.f;
            const bool have = valid && pre(ci, pd);
            const float* rowp = X + (int64_t)id * D;
            float sacc = 0.f;
            if (valid && !have)
#pragma unroll 4
                for (int c = r; c < D; c += 8) {
                    const float df = __fsub_rn(qs[c], __ldg(rowp + c));
                    sacc = __fmaf_rn(df, df, sacc);
                }
            const float t = __fadd_rn(sacc, __shfl_xor_sync(0xffffffffu, sacc, 4));
            const float u = __fadd_rn(t, __shfl_xor_sync(0xffffffffu, t, 2));
            const float v = __fadd_rn(u, __shfl_xor_sync(0xffffffffu, u, 1));
            dist = have ? pd : v;
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
}

// Visits every candidate id of query q: the ids of every matched bucket over
// all L tables and T probes, duplicates included (the reference's candidate
// lists, cuLSH_SearchTables.cu:321-343). The L*T bucket slots are read in
// chunks of CH by all NT threads at once (coalesced along t), the matched
// buckets compacted in shared memory with their sizes, and the ids of the
// chunk visited as one flattened range so that small and large buckets both
// keep every thread busy. f(id) is called once per (bucket, id) occurrence by
// some thread of the block; every thread must call this function.
struct BucketView {
    const int32_t* qbuckets;   // [L][Q*T]
    const uint64_t* boff;      // [L+1]
    const uint32_t* starts;
    const uint32_t* sizes;
    const uint32_t* ids;       // [L][N]
    int64_t N;
    int L, T, Q;
};

template <int NT, int CH>
struct GatherSmem {
    uint64_t base[CH];         // ids offset of each matched bucket
    unsigned long long pre[CH];  // inclusive prefix of the bucket sizes
    uint32_t n;
};

template <int NT, int CH, class F>
__device__ __forceinline__ void gather_bucket_ids(const BucketView& v, int q, GatherSmem<NT, CH>& g, F f) {
    const int tid = threadIdx.x, lane = tid & 31;
    const int T = v.T, LT = v.L * v.T;
    for (int c0 = 0; c0 < LT; c0 += CH) {
        if (tid == 0) g.n = 0;
        __syncthreads();
        const int c1 = min(LT, c0 + CH);
        for (int e = c0 + tid; e < c1; e += NT) {
            const int l = e / T, t = e - l * T;
            const int32_t j = __ldg(v.qbuckets + (int64_t)l * v.Q * T + (int64_t)q * T + t);
            if (j >= 0) {
                const uint64_t gi = __ldg(v.boff + l) + (uint32_t)j;
                const uint32_t st = __ldg(v.starts + gi), sz = __ldg(v.sizes + gi);
                if (sz) {
                    const uint32_t k = atomicAdd(&g.n, 1u);
                    g.base[k] = (uint64_t)l * (uint64_t)v.N + st;
                    g.pre[k] = sz;
                }
            }
        }
        __syncthreads();
        const uint32_t n = g.n;
        if (n == 0) continue;   // uniform: every thread read the same n
        if (tid < 32) {
            unsigned long long carry = 0;
            for (uint32_t b = 0; b < n; b += 32) {
                const uint32_t k = b + lane;
                unsigned long long x = k < n ? g.pre[k] : 0ull;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o) x += y;
                }
                if (k < n) g.pre[k] = x + carry;
                carry += __shfl_sync(0xffffffffu, x, 31);
            }
        }
        __syncthreads();
        const unsigned long long total = g.pre[n - 1];
        // h: first bucket whose inclusive prefix exceeds i. i only grows, so
        // h is kept between steps and searched for only when i leaves it.
        uint32_t h = 0;
        for (unsigned long long i = tid; i < total; i += NT) {
            if (g.pre[h] <= i) {
                uint32_t lo = h + 1, hi = n - 1;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (g.pre[mid] > i) hi = mid;
                    else lo = mid + 1;
                }
                h = lo;
            }
            const uint64_t off = i - (h ? g.pre[h - 1] : 0ull);
            f(__ldg(v.ids + g.base[h] + off));
        }
        __syncthreads();
    }
}

}  // namespace culsh
