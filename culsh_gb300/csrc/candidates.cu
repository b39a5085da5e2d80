// K4 (batched form): candidate gather / dedup / distance / top-K as one
// persistent work-stealing kernel.
//
// Same results as k_candidates (query.cu), organised for heavy-tailed
// candidate counts and for CUDA-graph capture (no host round trip):
//  * k_plan_items turns every query with C > 0 non-unique candidates into
//    P = min(64, ceil(C / chunk)) work items; item p of a query owns the
//    candidate ids whose hash h (32 bits) has floor(h * P / 2^32) = p, so the items of a query
//    deduplicate disjoint id sets (each fits the shared-memory set) and can be
//    processed by different CTAs. Queries without candidates get their padded
//    output ((-1, FLT_MAX) x K) right there.
//  * k_candidates_ws is a persistent grid that claims items with an atomic
//    counter (work stealing). Each item yields an exact top-K over its id
//    partition; the last item of a query to finish merges the P partial lists
//    (threadfence + arrival counter) into the final ascending (distance, id)
//    top-K. Distances follow the reference's lane order (cuLSH_Kernels.cu:301-348)
//    exactly as in k_candidates.
//  * A partition that does not fit the shared-memory set raises an overflow
//    count instead of spilling; the host then re-runs the search through the
//    arena-based kernel (rare: more than ~65k non-unique candidates for one
//    query).
#include <atomic>
#include <cfloat>

#include <cuda_bf16.h>

#include <algorithm>

#include "culsh_internal.cuh"
#include "topk_common.cuh"

namespace culsh {
namespace {

constexpr uint32_t kPartSalt = 0x5bd1e995u;
constexpr int GCH = 256;               // bucket slots scanned per gather chunk

constexpr int PT_PLAN = 256;           // queries per planning block

// One thread per query: partition count, a block scan, one atomic range
// reservation per block, so every query's items are contiguous.
__global__ void __launch_bounds__(PT_PLAN) k_plan_items(WsArgs a) {
    __shared__ uint32_t ws[PT_PLAN / 32];
    __shared__ uint32_t s_base;
    __shared__ uint8_t s_empty[PT_PLAN];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int q0 = blockIdx.x * PT_PLAN;
    const int q = q0 + tid < a.Q ? (a.order ? (int)a.order[q0 + tid] : q0 + tid) : a.Q;
    uint32_t P = 0;
    bool dense = false;
    if (q < a.Q) {
        const unsigned long long C = a.cnu[q];
        // near-exhaustive candidate sets go to the bitmap kernel instead
        dense = C >= a.dense_min;
        P = (C == 0 || dense) ? 0u : (uint32_t)min((unsigned long long)a.pmax, (C + a.chunk - 1) / a.chunk);
        if (dense) a.dense_q[atomicAdd(a.n_dense, 1u)] = q;
    }
    s_empty[tid] = q < a.Q && P == 0 && !dense;
    uint32_t x = P;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (tid == 0) {
        uint32_t t = 0;
        for (int i = 0; i < PT_PLAN / 32; ++i) {
            const uint32_t v = ws[i];
            ws[i] = t;
            t += v;
        }
        // More items than the partial-list buffers hold: the work-stealing
        // kernel then runs nothing and the host uses the per-query kernel.
        const uint32_t base = t ? atomicAdd(a.n_items, t) : 0u;
        if (t && (unsigned long long)base + t > a.item_cap) atomicOr(a.overflow, 1u);
        s_base = base;
    }
    __syncthreads();
    if (q < a.Q) {
        const uint32_t off = s_base + ws[w] + x - P;
        a.q_items[q] = (int)P;
        a.q_off[q] = (int)off;
        a.q_done[q] = 0;
        a.cu[q] = 0;
        for (uint32_t k = 0; k < P && off + k < a.item_cap; ++k) {
            a.item_q[off + k] = q;
            a.item_p[off + k] = (uint8_t)k;
        }
    }
    // Queries without candidates: padded output ((-1, FLT_MAX) x K), written
    // cooperatively so that the stores coalesce.
    const int nq = min(PT_PLAN, a.Q - q0);
    const int K = a.K;
    for (int i = tid; i < nq * K; i += PT_PLAN) {
        const int ql = i / K;
        if (s_empty[ql]) {
            const int64_t qq = a.order ? (int64_t)a.order[q0 + ql] : (int64_t)(q0 + ql);
            const int64_t o = qq * K + (i - ql * K);
            a.out_ids[o] = -1;
            a.out_d[o] = FLT_MAX;
        }
    }
}

// Locality order of the queries: a counting sort into kOrderBins bins of the
// home bucket of table 0 (bucket indices follow the lexicographic order of
// the codes, so nearby bins hold nearby points); queries without a home
// bucket go to the last bin. Order within a bin is arbitrary.
__device__ __forceinline__ uint32_t order_bin(const WsArgs& a, int q) {
    const int32_t b = a.qbuckets[(int64_t)q * a.T];   // table 0, probe 0
    const uint64_t b0 = a.boff[1] - a.boff[0];
    return b < 0 || b0 == 0 ? (uint32_t)kOrderBins : (uint32_t)((uint64_t)b * kOrderBins / b0);
}

__global__ void k_order_hist(WsArgs a) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < a.Q) atomicAdd(a.order_bins + order_bin(a, q), 1u);
}

// Exclusive scan of kOrderBins + 1 counters in one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_order_scan(WsArgs a) {
    constexpr int PER = (kOrderBins + 1 + 1023) / 1024;
    __shared__ uint32_t warp_sum[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    uint32_t v[PER], tot = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int i = tid * PER + k;
        v[k] = i <= kOrderBins ? a.order_bins[i] : 0u;
        tot += v[k];
    }
    uint32_t x = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t s = warp_sum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_sum[lane] = s - warp_sum[lane];
    }
    __syncthreads();
    uint32_t run = warp_sum[w] + x - tot;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int i = tid * PER + k;
        if (i <= kOrderBins) a.order_bins[i] = run;
        run += v[k];
    }
}

__global__ void k_order_scatter(WsArgs a) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < a.Q) a.order[atomicAdd(a.order_bins + order_bin(a, q), 1u)] = (uint32_t)q;
}

// WT threads per item: WT / 32 warps each keep a sorted top-K list over a
// strided share of the item's candidates (tuned: 64, 128, 256 or 512; wide
// items keep more row gathers in flight per block of shared memory).
// W_SLOTS: shared hash-set slots per item (4096, 8192 or 16384, tuned); an
// item holds at most W_CAP = W_SLOTS / 2 distinct ids. Every item of a query
// scans the query's whole id list and keeps its partition, so larger sets
// (fewer, larger partitions) scan less at the cost of occupancy.
template <int WT, bool kBF16, int W_SLOTS>
__global__ void __launch_bounds__(WT) k_candidates_ws(WsArgs a) {
    constexpr int WW = WT / 32;
    constexpr int W_CAP = W_SLOTS / 2;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t s_ucount;
    __shared__ int s_item, s_last, s_wn[WW];
    __shared__ GatherSmem<WT, GCH> s_gather;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int D = a.D, K = a.K, L = a.L, T = a.T;
    const int Dp = (D + 3) & ~3;
    float* qs = reinterpret_cast<float*>(smem);
    uint32_t* hset = reinterpret_cast<uint32_t*>(qs + Dp);
    uint32_t* ulist = hset + W_SLOTS;
    float* wd_all = reinterpret_cast<float*>(ulist + W_CAP);
    uint32_t* wi_all = reinterpret_cast<uint32_t*>(wd_all + WW * K);
    float* wd = wd_all + warp * K;
    uint32_t* wi = wi_all + warp * K;
    // BF16 form: approximate distance and error bound of each candidate.
    float* dA = reinterpret_cast<float*>(wi_all + WW * K);
    float* eA = dA + W_CAP;
    __shared__ float s_tau;
    __shared__ uint32_t s_scount, s_recheck, s_skip;
    // Bit 0 of the overflow word: the plan did not fit (set by k_plan_items,
    // which has finished). Read once and broadcast, so that the whole block
    // returns or none of it does; bit 1 (a set overflow) may be raised by
    // other blocks meanwhile and is left to the host.
    if (tid == 0) s_skip = *(volatile unsigned int*)a.overflow & 1u;
    __syncthreads();
    if (s_skip) return;
    const unsigned int n_items = *a.n_items;
    const bool vec = (D & 3) == 0;

    for (;;) {
        if (tid == 0) s_item = (int)atomicAdd(a.next_item, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= (int)n_items) break;
        const int q = a.item_q[item];
        const uint32_t p = a.item_p[item];
        const uint32_t P = (uint32_t)a.q_items[q];
        const unsigned long long C = a.cnu[q];
        for (int i = tid; i < Dp; i += WT) qs[i] = i < D ? a.queries[(int64_t)q * D + i] : 0.0f;
        for (int i = tid; i < W_SLOTS; i += WT) hset[i] = kEmpty32;
        if (tid == 0) s_ucount = 0;
        __syncthreads();

        // Gather this item's id partition from every matched bucket.
        const BucketView bv{a.qbuckets, a.boff, a.starts, a.sizes, a.ids, a.N, L, T, a.Q};
        gather_bucket_ids<WT, GCH>(bv, q, s_gather, [&](uint32_t id) {
            if (P > 1 && (uint32_t)(((uint64_t)mix32(id ^ kPartSalt) * P) >> 32) != p) return;
            set_insert(hset, W_SLOTS - 1, ulist, W_CAP, &s_ucount, id);
        });
        __syncthreads();
        uint32_t U = s_ucount;
        if (U > W_CAP) {   // the set overflowed: flag it, finish the protocol with no candidates
            if (tid == 0) atomicOr(a.overflow, 2u);
            U = 0;
        }

        // Exact FP32 distances in the reference lane order over list entries
        // [0, cnt) (entry j is ulist[idx_of(j)]), into per-warp sorted top-K
        // lists; an entry whose distance is already exact (pre) is not loaded.
        int n = 0;
        float thr_d = FLT_MAX;
        uint32_t thr_i = 0;
        auto fp32_pass = [&](uint32_t cnt, auto idx_of, auto pre) {
            fp32_dist_pass<WW>(a.X, D, qs, vec, cnt, idx_of, [&](uint32_t ci) { return ulist[ci]; }, pre, wd, wi, K,
                               n, thr_d, thr_i);
        };
        if constexpr (!kBF16) {
            fp32_pass(U, [](uint32_t j) { return j; }, [](uint32_t, float&) { return false; });
        } else {
            // Pass 1: BF16 rows. d~ is computed in the reference lane order
            // from the bf16 copy; E bounds |d~ - d| where d is the FP32
            // distance (exact rows: E = 0, since d~ is then d itself; rows
            // with extreme magnitudes: E = inf). Each warp keeps the K
            // smallest upper ends d~ + E; tau, the K-th smallest over the
            // item, caps the distance of its K nearest, so only candidates
            // with d~ - E <= tau can be among them.
            const int per = vec ? 16 : 4;
            for (uint32_t base = warp * per; base < U; base += WW * per) {
                float dt = 0.f, b1 = 0.f, b2 = 0.f;
                uint32_t ci, id;
                bool own;
                if (vec) {
                    ci = base + (lane >> 1);
                    const int h = lane & 1;
                    const bool valid = ci < U;
                    id = valid ? ulist[ci] : 0u;
                    const uint16_t* rowp = a.xb + (int64_t)id * D;
                    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
                    if (valid) {
#pragma unroll 8
                        for (int c = 4 * h; c < D; c += 8) {
                            const uint2 raw = __ldg(reinterpret_cast<const uint2*>(rowp + c));
                            const float x0 = __uint_as_float(raw.x << 16), x1 = __uint_as_float(raw.x & 0xFFFF0000u);
                            const float x2 = __uint_as_float(raw.y << 16), x3 = __uint_as_float(raw.y & 0xFFFF0000u);
                            const float4 qv = *reinterpret_cast<const float4*>(qs + c);
                            const float d0 = __fsub_rn(qv.x, x0), d1 = __fsub_rn(qv.y, x1);
                            const float d2 = __fsub_rn(qv.z, x2), d3 = __fsub_rn(qv.w, x3);
                            s0 = __fmaf_rn(d0, d0, s0);
                            s1 = __fmaf_rn(d1, d1, s1);
                            s2 = __fmaf_rn(d2, d2, s2);
                            s3 = __fmaf_rn(d3, d3, s3);
                            b1 = __fmaf_rn(fabsf(x0), fabsf(d0), b1);
                            b1 = __fmaf_rn(fabsf(x1), fabsf(d1), b1);
                            b1 = __fmaf_rn(fabsf(x2), fabsf(d2), b1);
                            b1 = __fmaf_rn(fabsf(x3), fabsf(d3), b1);
                            b2 = __fmaf_rn(x0, x0, b2);
                            b2 = __fmaf_rn(x1, x1, b2);
                            b2 = __fmaf_rn(x2, x2, b2);
                            b2 = __fmaf_rn(x3, x3, b2);
                        }
                    }
                    const float o0 = __shfl_xor_sync(0xffffffffu, s0, 1), o1 = __shfl_xor_sync(0xffffffffu, s1, 1);
                    const float o2 = __shfl_xor_sync(0xffffffffu, s2, 1), o3 = __shfl_xor_sync(0xffffffffu, s3, 1);
                    const float t0 = __fadd_rn(s0, o0), t1 = __fadd_rn(s1, o1), t2 = __fadd_rn(s2, o2),
                                t3 = __fadd_rn(s3, o3);
                    dt = __fadd_rn(__fadd_rn(t0, t2), __fadd_rn(t1, t3));
                    b1 = __fadd_rn(b1, __shfl_xor_sync(0xffffffffu, b1, 1));
                    b2 = __fadd_rn(b2, __shfl_xor_sync(0xffffffffu, b2, 1));
                    own = valid && h == 0;
                } else {
                    ci = base + (lane >> 3);
                    const int r = lane & 7;
                    const bool valid = ci < U;
                    id = valid ? ulist[ci] : 0u;
                    const uint16_t* rowp = a.xb + (int64_t)id * D;
                    float sacc = 0.f;
                    if (valid)
#pragma unroll 4
                        for (int c = r; c < D; c += 8) {
                            const float x = __uint_as_float((uint32_t)__ldg(rowp + c) << 16);
                            const float df = __fsub_rn(qs[c], x);
                            sacc = __fmaf_rn(df, df, sacc);
                            b1 = __fmaf_rn(fabsf(x), fabsf(df), b1);
                            b2 = __fmaf_rn(x, x, b2);
                        }
                    const float t = __fadd_rn(sacc, __shfl_xor_sync(0xffffffffu, sacc, 4));
                    const float u = __fadd_rn(t, __shfl_xor_sync(0xffffffffu, t, 2));
                    dt = __fadd_rn(u, __shfl_xor_sync(0xffffffffu, u, 1));
#pragma unroll
                    for (int o = 4; o > 0; o >>= 1) {
                        b1 = __fadd_rn(b1, __shfl_xor_sync(0xffffffffu, b1, o));
                        b2 = __fadd_rn(b2, __shfl_xor_sync(0xffffffffu, b2, o));
                    }
                    own = valid && r == 0;
                }
                float e = 0.f, up = 0.f;
                if (own) {
                    const uint8_t fl = __ldg(a.xflag + id);
                    if (fl == 1) {
                        e = 0.f;
                    } else if (fl == 2 || !(dt <= FLT_MAX)) {
                        e = __int_as_float(0x7f800000);
                    } else {
                        // E = c1 * d~ + c2 * (2 rho b1 + rho^2 b2), upward roundings
                        const float rho = 0.00393676758f;   // 2^-8 (1 + 2^-7), bf16 rounding relative to |x~|
                        const float delta = __fmaf_ru(rho * rho, b2, __fmul_ru(2.0f * rho, b1));
                        e = __fmaf_ru(a.e_c1, dt, __fmul_ru(a.e_c2, delta));
                    }
                    dA[ci] = dt;
                    eA[ci] = e;
                    up = __fadd_ru(dt, e);
                }
                uint32_t want = __ballot_sync(0xffffffffu, own && lessp(up, ci, thr_d, thr_i));
                while (want) {
                    const int src = __ffs(want) - 1;
                    want &= want - 1;
                    const float cdv = __shfl_sync(0xffffffffu, up, src);
                    const uint32_t cid = __shfl_sync(0xffffffffu, ci, src);
                    if (lessp(cdv, cid, thr_d, thr_i)) warp_insert(wd, wi, n, K, cdv, cid, thr_d, thr_i);
                }
            }
            if (lane == 0) s_wn[warp] = n;
            if (tid == 0) s_scount = s_recheck = 0;
            __syncthreads();
            if (warp == 0) {
                for (int w = 1; w < WW; ++w) {
                    const int nw = s_wn[w];
                    for (int e = 0; e < nw; ++e) {
                        const float d = wd_all[w * K + e];
                        const uint32_t id = wi_all[w * K + e];
                        if (!lessp(d, id, thr_d, thr_i)) break;
                        warp_insert(wd, wi, n, K, d, id, thr_d, thr_i);
                    }
                }
                if (lane == 0) s_tau = n == K ? wd[K - 1] : __int_as_float(0x7f800000);
            }
            __syncthreads();
            // Shortlist (into the free hash-set memory): d~ - E <= tau.
            const float tau = s_tau;
            uint32_t* slist = hset;
            uint32_t rc = 0;
            for (uint32_t ci = tid; ci < U; ci += WT)
                if (__fsub_rd(dA[ci], eA[ci]) <= tau) {
                    slist[atomicAdd(&s_scount, 1u)] = ci;
                    rc += eA[ci] != 0.f;
                }
            if (rc) atomicAdd(&s_recheck, rc);
            __syncthreads();
            if (tid == 0 && s_recheck) atomicAdd(a.rechecked, (unsigned long long)s_recheck);
            // Pass 2: exact distances of the shortlist (re-read in FP32 only
            // for rows whose bf16 copy is inexact).
            n = 0;
            thr_d = FLT_MAX;
            thr_i = 0;
            fp32_pass(s_scount, [&](uint32_t j) { return slist[j]; }, [&](uint32_t ci, float& d) {
                if (eA[ci] != 0.f) return false;
                d = dA[ci];
                return true;
            });
        }
        if (lane == 0) s_wn[warp] = n;
        __syncthreads();
        if (warp == 0) {
            for (int w = 1; w < WW; ++w) {
                const int nw = s_wn[w];
                for (int e = 0; e < nw; ++e) {
                    const float d = wd_all[w * K + e];
                    const uint32_t id = wi_all[w * K + e];
                    if (!lessp(d, id, thr_d, thr_i)) break;
                    warp_insert(wd, wi, n, K, d, id, thr_d, thr_i);
                }
            }
            if (lane == 0) {
                atomicAdd(a.cu + q, (unsigned long long)U);
                atomicAdd(a.totals + 0, (unsigned long long)U);
            }
        }
        if (P == 1) {
            if (warp == 0) {
                int32_t* oid = a.out_ids + (int64_t)q * K;
                float* od = a.out_d + (int64_t)q * K;
                for (int k = lane; k < K; k += 32) {
                    oid[k] = k < n ? (int32_t)wi[k] : -1;
                    od[k] = k < n ? wd[k] : FLT_MAX;
                }
                if (lane == 0) atomicAdd(a.totals + 1, C);
            }
        } else {
            // Publish this partition's list; the last partition to finish merges.
            if (warp == 0) {
                float* pd = a.part_d + (int64_t)item * K;
                uint32_t* pi = a.part_i + (int64_t)item * K;
                for (int k = lane; k < n; k += 32) {
                    pd[k] = wd[k];
                    pi[k] = wi[k];
                }
                if (lane == 0) a.part_n[item] = n;
                __threadfence();
                __syncwarp();
                if (lane == 0) s_last = atomicAdd(a.q_done + q, 1u) == P - 1;
                __syncwarp();
                if (s_last) {
                    __threadfence();
                    n = 0;
                    thr_d = FLT_MAX;
                    thr_i = 0;
                    const int first = a.q_off[q];
                    for (uint32_t k = 0; k < P; ++k) {
                        const int it = first + (int)k;
                        const int m = *(volatile const int*)(a.part_n + it);
                        const float* pd2 = a.part_d + (int64_t)it * K;
                        const uint32_t* pi2 = a.part_i + (int64_t)it * K;
                        for (int e = 0; e < m; ++e) {
                            const float d = *(volatile const float*)(pd2 + e);
                            const uint32_t id = *(volatile const uint32_t*)(pi2 + e);
                            if (!lessp(d, id, thr_d, thr_i)) break;
                            warp_insert(wd, wi, n, K, d, id, thr_d, thr_i);
                        }
                    }
                    int32_t* oid = a.out_ids + (int64_t)q * K;
                    float* od = a.out_d + (int64_t)q * K;
                    for (int k = lane; k < K; k += 32) {
                        oid[k] = k < n ? (int32_t)wi[k] : -1;
                        od[k] = k < n ? wd[k] : FLT_MAX;
                    }
                    if (lane == 0) atomicAdd(a.totals + 1, C);
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace

// Dense form: a query whose non-unique candidates reach dense_min (a large
// share of the dataset) is deduplicated in an N-bit bitmap in shared memory
// rather than in id partitions; the bitmap is then compacted 8,192 bits at a
// time into a candidate list for the exact distance pass. Persistent grid,
// one query per CTA at a time.
constexpr int DT = 256;
constexpr int DW = DT / 32;

__global__ void __launch_bounds__(DT, 1) k_candidates_dense(WsArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ GatherSmem<DT, GCH> s_gather;
    __shared__ int s_q;
    __shared__ uint32_t s_ws[DW], s_wn[DW];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int D = a.D, K = a.K, L = a.L, T = a.T;
    const int Dp = (D + 3) & ~3;
    const uint32_t nwords = (uint32_t)((a.N + 31) >> 5);
    const uint32_t nwp = (nwords + 3) & ~3u;
    float* qs = reinterpret_cast<float*>(smem);
    uint32_t* bits = reinterpret_cast<uint32_t*>(qs + Dp);
    uint32_t* clist = bits + nwp;                       // DT * 32 candidate ids
    float* wd_all = reinterpret_cast<float*>(clist + DT * 32);
    uint32_t* wi_all = reinterpret_cast<uint32_t*>(wd_all + DW * K);
    float* wd = wd_all + warp * K;
    uint32_t* wi = wi_all + warp * K;
    const bool vec = (D & 3) == 0;
    const unsigned int ndense = *a.n_dense;

    for (;;) {
        if (tid == 0) {
            const unsigned int k = atomicAdd(a.dense_next, 1u);
            s_q = k < ndense ? a.dense_q[k] : -1;
        }
        __syncthreads();
        const int q = s_q;
        if (q < 0) break;
        for (int i = tid; i < Dp; i += DT) qs[i] = i < D ? a.queries[(int64_t)q * D + i] : 0.0f;
        for (uint32_t i = tid; i < nwords; i += DT) bits[i] = 0u;
        __syncthreads();
        const BucketView bv{a.qbuckets, a.boff, a.starts, a.sizes, a.ids, a.N, L, T, a.Q};
        gather_bucket_ids<DT, GCH>(bv, q, s_gather,
                                   [&](uint32_t id) { atomicOr(&bits[id >> 5], 1u << (id & 31)); });
        __syncthreads();

        int n = 0;
        float thr_d = FLT_MAX;
        uint32_t thr_i = 0;
        unsigned long long U = 0;   // unique candidates (summed by every thread alike)
        for (uint32_t w0 = 0; w0 < nwords; w0 += DT) {
            const uint32_t w = w0 + tid;
            const uint32_t word = w < nwords ? bits[w] : 0u;
            // block exclusive scan of the set-bit counts
            const uint32_t c = __popc(word);
            uint32_t x = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) s_ws[warp] = x;
            __syncthreads();
            uint32_t before = 0, total = 0;
            for (int i = 0; i < DW; ++i) {
                const uint32_t v = s_ws[i];
                before += i < warp ? v : 0u;
                total += v;
            }
            uint32_t k = before + x - c;
            for (uint32_t m = word; m; m &= m - 1) clist[k++] = w * 32 + (uint32_t)(__ffs((int)m) - 1);
            __syncthreads();
            fp32_dist_pass<DW>(a.X, D, qs, vec, total, [](uint32_t j) { return j; },
                               [&](uint32_t ci) { return clist[ci]; }, [](uint32_t, float&) { return false; }, wd,
                               wi, K, n, thr_d, thr_i);
            U += total;
            __syncthreads();
        }
        if (lane == 0) s_wn[warp] = n;
        __syncthreads();
        if (warp == 0) {
            for (int ww = 1; ww < DW; ++ww) {
                const int nw = s_wn[ww];
                for (int e = 0; e < nw; ++e) {
                    const float d = wd_all[ww * K + e];
                    const uint32_t id = wi_all[ww * K + e];
                    if (!lessp(d, id, thr_d, thr_i)) break;
                    warp_insert(wd, wi, n, K, d, id, thr_d, thr_i);
                }
            }
            int32_t* oid = a.out_ids + (int64_t)q * K;
            float* od = a.out_d + (int64_t)q * K;
            for (int k2 = lane; k2 < K; k2 += 32) {
                oid[k2] = k2 < n ? (int32_t)wi[k2] : -1;
                od[k2] = k2 < n ? wd[k2] : FLT_MAX;
            }
            if (lane == 0) {
                a.cu[q] = U;
                atomicAdd(a.totals + 0, U);
                atomicAdd(a.totals + 1, a.cnu[q]);
            }
        }
        __syncthreads();
    }
}

// Membership rows of the dense queries for the tensor-core path
// (knn_tc.cu): query k of the dense list gets row bm[k][0 .. nwp) with bit i
// set when point i is one of its candidates (nwp - ceil(N/32) padding words
// stay zero). The bits are set in an N-bit bitmap in shared memory from the
// query's bucket ids (every matched bucket over the L tables and T probes,
// as the reference's candidate lists, cuLSH_SearchTables.cu:321-364) and
// copied out once; their count is the query's unique candidate count.
// Persistent grid, one query per CTA at a time, 1024 threads. The matched
// buckets are cut into units of at most BSEG consecutive ids; warp w takes
// units w, w + 32, ..., loads 32 x BU ids at a time (coalesced: a bucket's
// ids are contiguous, BU loads in flight per lane) and ORs their bits in.
// A matched bucket that has a bucket row (a.big_rows; up to BROWS of them
// per query) sets no bits: its row is ORed into the words as they are copied
// out, which replaces one shared-memory atomic per id by one 16-byte load
// per four words. The set is the same either way.
constexpr int BT = 1024;
constexpr int BU = 8;
constexpr uint32_t BSEG = 1024;
constexpr int BCH = 256;   // (table, probe) slots per compaction chunk
constexpr uint32_t BROWS = 64;

struct BitmapSmem {
    uint64_t base[BCH];     // ids offset of each matched bucket
    uint32_t size[BCH];
    uint32_t upre[BCH + 1]; // units before each matched bucket
    uint32_t n;
    uint32_t nrow;          // matched buckets with a bucket row (may exceed BROWS)
    uint32_t row[BROWS];    // their rows
};

// Row of global bucket gi among the n ascending bucket numbers of big_gi, -1
// if it has none.
__device__ __forceinline__ int big_row(const uint64_t* __restrict__ big_gi, int n, uint64_t gi) {
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const uint64_t v = __ldg(big_gi + mid);
        if (v == gi) return mid;
        if (v < gi) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

__global__ void __launch_bounds__(BT, 1) k_cand_bitmap(WsArgs a, uint32_t* __restrict__ bm, int nwp) {
    extern __shared__ __align__(16) uint32_t bits[];
    __shared__ BitmapSmem g;
    __shared__ int s_q, s_k;
    __shared__ unsigned long long s_cnt[BT / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = BT / 32;
    const unsigned int ndense = *a.n_dense;
    const int T = a.T, LT = a.L * a.T;
    // Thread 0 claims the next query while the block works on the current
    // one (the claim's round trip overlaps the work) and publishes it at the
    // end of the query, before the block's last barrier.
    if (tid == 0) {
        const unsigned int k = atomicAdd(a.dense_next, 1u);
        s_k = (int)k;
        s_q = k < ndense ? a.dense_q[k] : -1;
    }
    __syncthreads();
    for (;;) {
        const int q = s_q, k = s_k;
        if (q < 0) break;
        unsigned int knext = 0;
        if (tid == 0) knext = atomicAdd(a.dense_next, 1u);
        for (int i = tid * 4; i < nwp; i += BT * 4) *reinterpret_cast<uint4*>(bits + i) = make_uint4(0u, 0u, 0u, 0u);
        for (int c0 = 0; c0 < LT; c0 += BCH) {
            // matched buckets of this chunk of (table, probe) slots, with sizes
            if (tid == 0) {
                g.n = 0;
                if (c0 == 0) g.nrow = 0;
            }
            __syncthreads();
            const int c1 = min(LT, c0 + BCH);
            for (int e = c0 + tid; e < c1; e += BT) {
                const int l = e / T, t = e - l * T;
                const int32_t j = __ldg(a.qbuckets + (int64_t)l * a.Q * T + (int64_t)q * T + t);
                if (j >= 0) {
                    const uint64_t gi = __ldg(a.boff + l) + (uint32_t)j;
                    const uint32_t st = __ldg(a.starts + gi), sz = __ldg(a.sizes + gi);
                    if (a.nbig > 0 && sz >= a.big_min) {
                        const int r = big_row(a.big_gi, a.nbig, gi);
                        if (r >= 0) {
                            const uint32_t kr = atomicAdd(&g.nrow, 1u);
                            if (kr < BROWS) {
                                g.row[kr] = (uint32_t)r;
                                continue;
                            }
                        }
                    }
                    if (sz) {
                        const uint32_t kk = atomicAdd(&g.n, 1u);
                        g.base[kk] = (uint64_t)l * (uint64_t)a.N + st;
                        g.size[kk] = sz;
                    }
                }
            }
            __syncthreads();
            const uint32_t n = g.n;
            if (n == 0) continue;   // uniform
            if (warp == 0) {
                // exclusive scan of the units per bucket
                uint32_t carry = 0;
                for (uint32_t b0 = 0; b0 < n; b0 += 32) {
                    const uint32_t kk = b0 + lane;
                    const uint32_t c = kk < n ? (g.size[kk] + BSEG - 1) / BSEG : 0u;
                    uint32_t x = c;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                        if (lane >= o) x += y;
                    }
                    if (kk < n) g.upre[kk] = carry + x - c;
                    carry += __shfl_sync(0xffffffffu, x, 31);
                }
                if (lane == 0) g.upre[n] = carry;
            }
            __syncthreads();
            const uint32_t units = g.upre[n];
            for (uint32_t u = warp; u < units; u += NW) {
                // bucket of unit u: the last b with upre[b] <= u
                uint32_t lo = 0, hi = n - 1;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi + 1) >> 1;
                    if (g.upre[mid] <= u) lo = mid;
                    else hi = mid - 1;
                }
                const uint32_t off = (u - g.upre[lo]) * BSEG;
                const uint32_t cnt = min(BSEG, g.size[lo] - off);
                const uint32_t* src = a.ids + g.base[lo] + off;
                uint32_t j0 = 0;
                for (; j0 + 32 * BU <= cnt; j0 += 32 * BU) {   // full blocks: BU loads in flight per lane
                    uint32_t v[BU];
#pragma unroll
                    for (int b = 0; b < BU; ++b) v[b] = __ldg(src + j0 + b * 32 + lane);
#pragma unroll
                    for (int b = 0; b < BU; ++b) atomicOr(&bits[v[b] >> 5], 1u << (v[b] & 31));
                }
                for (; j0 < cnt; j0 += 32) {
                    const uint32_t j = j0 + lane;
                    if (j < cnt) {
                        const uint32_t v = __ldg(src + j);
                        atomicOr(&bits[v >> 5], 1u << (v & 31));
                    }
                }
            }
            __syncthreads();
        }
        uint32_t* row = bm + (int64_t)k * nwp;
        const uint32_t nrow = min(g.nrow, BROWS);
        unsigned long long cnt = 0;
        for (int i = tid * 4; i < nwp; i += BT * 4) {
            uint4 v = *reinterpret_cast<const uint4*>(bits + i);
#pragma unroll 4
            for (uint32_t r = 0; r < nrow; ++r) {
                const uint4 w = __ldg(reinterpret_cast<const uint4*>(a.big_rows + (size_t)g.row[r] * nwp + i));
                v.x |= w.x;
                v.y |= w.y;
                v.z |= w.z;
                v.w |= w.w;
            }
            *reinterpret_cast<uint4*>(row + i) = v;
            cnt += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if (lane == 0) s_cnt[warp] = cnt;
        __syncthreads();
        if (tid == 0) {
            unsigned long long U = 0;
            for (int w = 0; w < NW; ++w) U += s_cnt[w];
            a.cu[q] = U;
            atomicAdd(a.totals + 0, U);
            atomicAdd(a.totals + 1, a.cnu[q]);
            s_k = (int)knext;
            s_q = knext < ndense ? a.dense_q[knext] : -1;
        }
        __syncthreads();
    }
}

size_t bitmap_smem_bytes(int64_t N) { return 4 * (size_t)((((N + 31) >> 5) + 3) & ~3ll); }

__global__ void k_big_find(const uint32_t* __restrict__ sizes, uint64_t totB, uint32_t big_min, uint64_t* gi,
                           uint32_t* sz, unsigned int* cnt, unsigned int cap) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < totB; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = sizes[i];
        if (s >= big_min) {
            const unsigned int k = atomicAdd(cnt, 1u);
            if (k < cap) {
                gi[k] = i;
                sz[k] = s;
            }
        }
    }
}

// Row r (blockIdx.y) gets the bits of bucket gi[r]'s ids (table tl[r]).
__global__ void k_big_fill(const uint64_t* __restrict__ gi, const int32_t* __restrict__ tl,
                           const uint32_t* __restrict__ starts, const uint32_t* __restrict__ sizes,
                           const uint32_t* __restrict__ ids, int64_t N, uint32_t* rows, int nwp) {
    const int r = blockIdx.y;
    const uint64_t b = gi[r];
    const uint32_t st = starts[b], sz = sizes[b];
    const uint32_t* src = ids + (uint64_t)tl[r] * N + st;
    uint32_t* row = rows + (size_t)r * nwp;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < sz; j += gridDim.x * blockDim.x) {
        const uint32_t v = src[j];
        atomicOr(row + (v >> 5), 1u << (v & 31));
    }
}

cudaError_t launch_big_find(const uint32_t* sizes, uint64_t totB, uint32_t big_min, uint64_t* gi, uint32_t* sz,
                            unsigned int* cnt, unsigned int cap, cudaStream_t st) {
    if (totB == 0) return cudaSuccess;
    const unsigned g = (unsigned)std::min<uint64_t>((totB + 255) / 256, 4096);
    k_big_find<<<g, 256, 0, st>>>(sizes, totB, big_min, gi, sz, cnt, cap);
    return cudaGetLastError();
}

cudaError_t launch_big_fill(const uint64_t* gi, const int32_t* tl, int nbig, const uint32_t* starts,
                            const uint32_t* sizes, const uint32_t* ids, int64_t N, uint32_t* rows, int nwp,
                            cudaStream_t st) {
    if (nbig <= 0) return cudaSuccess;
    k_big_fill<<<dim3(16, (unsigned)nbig), 256, 0, st>>>(gi, tl, starts, sizes, ids, N, rows, nwp);
    return cudaGetLastError();
}

cudaError_t launch_cand_bitmap(const WsArgs& a, uint32_t* bm, int nwp, int grid, cudaStream_t st) {
    static std::atomic<size_t> cap{0};
    const size_t smem = 4 * (size_t)nwp;
    const cudaError_t e = opt_in_smem(k_cand_bitmap, smem, cap);
    if (e != cudaSuccess) return e;
    k_cand_bitmap<<<grid, BT, smem, st>>>(a, bm, nwp);
    return cudaGetLastError();
}

size_t dense_smem_bytes(int64_t N, int D, int K) {
    const size_t nwp = (size_t)((((N + 31) >> 5) + 3) & ~3ll);
    return sizeof(float) * (size_t)((D + 3) & ~3) + 4 * nwp + 4 * (size_t)DT * 32 +
           (size_t)DW * K * (sizeof(float) + sizeof(uint32_t));
}

size_t ws_smem_bytes(int D, int K, int wt, int bf16, int slots) {
    const size_t cap = (size_t)slots / 2;
    return sizeof(float) * (size_t)((D + 3) & ~3) + sizeof(uint32_t) * ((size_t)slots + cap) +
           (size_t)(wt / 32) * K * (sizeof(float) + sizeof(uint32_t)) + (bf16 ? 2 * sizeof(float) * cap : 0);
}

cudaError_t launch_order_queries(const WsArgs& a, cudaStream_t st) {
    if (a.Q <= 0 || !a.order) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(a.order_bins, 0, sizeof(uint32_t) * (kOrderBins + 1), st);
    if (e != cudaSuccess) return e;
    const unsigned g = (unsigned)((a.Q + 255) / 256);
    k_order_hist<<<g, 256, 0, st>>>(a);
    k_order_scan<<<1, 1024, 0, st>>>(a);
    k_order_scatter<<<g, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_plan_items(const WsArgs& a, cudaStream_t st) {
    if (a.Q <= 0) return cudaSuccess;
    k_plan_items<<<(a.Q + PT_PLAN - 1) / PT_PLAN, PT_PLAN, 0, st>>>(a);
    return cudaGetLastError();
}

namespace {
template <int WT, bool kBF16, int SL>
std::atomic<size_t>& ws_smem_cap() {
    static std::atomic<size_t> cap{0};   // dynamic shared memory this kernel is opted into
    return cap;
}

template <int WT, bool kBF16, int SL>
cudaError_t launch_ws_v(const WsArgs& a, int grid, cudaStream_t st) {
    const size_t smem = ws_smem_bytes(a.D, a.K, WT, kBF16, SL);
    const cudaError_t e = opt_in_smem(k_candidates_ws<WT, kBF16, SL>, smem, ws_smem_cap<WT, kBF16, SL>());
    if (e != cudaSuccess) return e;
    k_candidates_ws<WT, kBF16, SL><<<grid, WT, smem, st>>>(a);
    return cudaGetLastError();
}

template <int WT, bool kBF16, int SL>
int ws_bps_v(int D, int K) {
    int n = 0;
    const size_t smem = ws_smem_bytes(D, K, WT, kBF16, SL);
    if (opt_in_smem(k_candidates_ws<WT, kBF16, SL>, smem, ws_smem_cap<WT, kBF16, SL>()) != cudaSuccess) return 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_candidates_ws<WT, kBF16, SL>, WT, smem) != cudaSuccess)
        n = 1;
    return n > 0 ? n : 1;
}

template <bool kBF16, int SL>
cudaError_t launch_ws_w(const WsArgs& a, int grid, cudaStream_t st) {
    switch (a.wt) {
        case 64: return launch_ws_v<64, kBF16, SL>(a, grid, st);
        case 256: return launch_ws_v<256, kBF16, SL>(a, grid, st);
        case 512: return launch_ws_v<512, kBF16, SL>(a, grid, st);
        default: return launch_ws_v<128, kBF16, SL>(a, grid, st);
    }
}

template <bool kBF16, int SL>
int ws_bps_w(int D, int K, int wt) {
    switch (wt) {
        case 64: return ws_bps_v<64, kBF16, SL>(D, K);
        case 256: return ws_bps_v<256, kBF16, SL>(D, K);
        case 512: return ws_bps_v<512, kBF16, SL>(D, K);
        default: return ws_bps_v<128, kBF16, SL>(D, K);
    }
}

// BF16 copy of the dataset (round to nearest even) and a per-row flag:
// 1 when every element is exact in bf16, 2 when a nonzero element has a
// magnitude outside [2^-100, 2^100] (the search then always re-checks the
// row in FP32), 0 otherwise. One warp per row.
__global__ void k_bf16_rows(const float* __restrict__ X, int64_t N, int D, uint16_t* __restrict__ xb,
                            uint8_t* __restrict__ flag) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = w0; r < N; r += nw) {
        bool exact = true, special = false;
        for (int d = lane; d < D; d += 32) {
            const float x = __ldg(X + r * D + d);
            const uint16_t h = __bfloat16_as_ushort(__float2bfloat16_rn(x));
            xb[r * D + d] = h;
            exact &= __uint_as_float((uint32_t)h << 16) == x;
            const float ax = fabsf(x);
            special |= x != 0.0f && !(ax >= 7.88860905e-31f && ax <= 1.26765060e30f);
        }
        exact = __all_sync(0xffffffffu, exact);
        special = __any_sync(0xffffffffu, special);
        if (lane == 0) flag[r] = special ? 2 : (exact ? 1 : 0);
    }
}
}  // namespace

cudaError_t launch_candidates_ws(const WsArgs& a, int grid, cudaStream_t st) {
    if (a.slots == 16384)
        return a.bf16 ? launch_ws_w<true, 16384>(a, grid, st) : launch_ws_w<false, 16384>(a, grid, st);
    if (a.slots == 8192) return a.bf16 ? launch_ws_w<true, 8192>(a, grid, st) : launch_ws_w<false, 8192>(a, grid, st);
    return a.bf16 ? launch_ws_w<true, 4096>(a, grid, st) : launch_ws_w<false, 4096>(a, grid, st);
}

int ws_blocks_per_sm(int D, int K, int wt, int bf16, int slots) {
    if (slots == 16384) return bf16 ? ws_bps_w<true, 16384>(D, K, wt) : ws_bps_w<false, 16384>(D, K, wt);
    if (slots == 8192) return bf16 ? ws_bps_w<true, 8192>(D, K, wt) : ws_bps_w<false, 8192>(D, K, wt);
    return bf16 ? ws_bps_w<true, 4096>(D, K, wt) : ws_bps_w<false, 4096>(D, K, wt);
}

cudaError_t launch_candidates_dense(const WsArgs& a, int grid, cudaStream_t st) {
    static std::atomic<size_t> cap{0};   // dynamic shared memory this kernel is opted into
    const size_t smem = dense_smem_bytes(a.N, a.D, a.K);
    const cudaError_t e = opt_in_smem(k_candidates_dense, smem, cap);
    if (e != cudaSuccess) return e;
    k_candidates_dense<<<grid, DT, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_bf16_rows(const float* X, int64_t N, int D, uint16_t* xb, uint8_t* flag, cudaStream_t st) {
    if (N <= 0) return cudaSuccess;
    const int64_t warps = std::min<int64_t>(N, 152 * 64);
    k_bf16_rows<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, st>>>(X, N, D, xb, flag);
    return cudaGetLastError();
}

}  // namespace culsh
