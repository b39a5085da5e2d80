// K4 (batched form): candidate gather / dedup / distance / top-K as one
// persistent work-stealing kernel.
//
// Same results as k_candidates (query.cu), organised for heavy-tailed
// candidate counts and for CUDA-graph capture (no host round trip):
//  * k_plan_items turns every query with C > 0 non-unique candidates into
//    P = min(64, ceil(C / 1024)) work items; item p of a query owns the
//    candidate ids whose hash falls in partition p, so the items of a query
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

#include "culsh_internal.cuh"
#include "topk_common.cuh"

namespace culsh {
namespace {

constexpr int W_SLOTS = 4096;          // shared hash slots per item
constexpr int W_CAP = W_SLOTS / 2;     // distinct ids per item
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
    const int q = q0 + tid;
    uint32_t P = 0;
    if (q < a.Q) {
        const unsigned long long C = a.cnu[q];
        P = C == 0 ? 0u : (uint32_t)min((unsigned long long)a.pmax, (C + a.chunk - 1) / a.chunk);
    }
    s_empty[tid] = q < a.Q && P == 0;
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
            a.out_ids[(int64_t)q0 * K + i] = -1;
            a.out_d[(int64_t)q0 * K + i] = FLT_MAX;
        }
    }
}

// WT threads per item: WT / 32 warps each keep a sorted top-K list over a
// strided share of the item's candidates (tuned: 64, 128 or 256).
template <int WT>
__global__ void __launch_bounds__(WT) k_candidates_ws(WsArgs a) {
    constexpr int WW = WT / 32;
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
    if (*(volatile unsigned int*)a.overflow) return;   // the plan did not fit
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
            if (P > 1 && mix32(id ^ kPartSalt) % P != p) return;
            set_insert(hset, W_SLOTS - 1, ulist, W_CAP, &s_ucount, id);
        });
        __syncthreads();
        uint32_t U = s_ucount;
        if (U > W_CAP) {   // the set overflowed: flag it, finish the protocol with no candidates
            if (tid == 0) atomicAdd(a.overflow, 1u);
            U = 0;
        }

        // Distances in the reference lane order, per-warp sorted top-K.
        int n = 0;
        float thr_d = FLT_MAX;
        uint32_t thr_i = 0;
        const int per = vec ? 16 : 4;
        for (uint32_t base = warp * per; base < U; base += WW * per) {
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
                const float t0 = __fadd_rn(s0, o0), t1 = __fadd_rn(s1, o1), t2 = __fadd_rn(s2, o2),
                            t3 = __fadd_rn(s3, o3);
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

size_t ws_smem_bytes(int D, int K, int wt) {
    return sizeof(float) * (size_t)((D + 3) & ~3) + sizeof(uint32_t) * (W_SLOTS + W_CAP) +
           (size_t)(wt / 32) * K * (sizeof(float) + sizeof(uint32_t));
}

cudaError_t launch_plan_items(const WsArgs& a, cudaStream_t st) {
    if (a.Q <= 0) return cudaSuccess;
    k_plan_items<<<(a.Q + PT_PLAN - 1) / PT_PLAN, PT_PLAN, 0, st>>>(a);
    return cudaGetLastError();
}

namespace {
template <int WT>
cudaError_t launch_ws_v(const WsArgs& a, int grid, cudaStream_t st) {
    const size_t smem = ws_smem_bytes(a.D, a.K, WT);
    static std::atomic<size_t> configured{0};   // largest dynamic shared memory opted into
    if (smem > 48 * 1024 && smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(k_candidates_ws<WT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    k_candidates_ws<WT><<<grid, WT, smem, st>>>(a);
    return cudaGetLastError();
}

template <int WT>
int ws_bps_v(int D, int K) {
    int n = 0;
    const size_t smem = ws_smem_bytes(D, K, WT);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_candidates_ws<WT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_candidates_ws<WT>, WT, smem) != cudaSuccess) n = 1;
    return n > 0 ? n : 1;
}
}  // namespace

cudaError_t launch_candidates_ws(const WsArgs& a, int grid, cudaStream_t st) {
    switch (a.wt) {
        case 64: return launch_ws_v<64>(a, grid, st);
        case 256: return launch_ws_v<256>(a, grid, st);
        default: return launch_ws_v<128>(a, grid, st);
    }
}

int ws_blocks_per_sm(int D, int K, int wt) {
    switch (wt) {
        case 64: return ws_bps_v<64>(D, K);
        case 256: return ws_bps_v<256>(D, K);
        default: return ws_bps_v<128>(D, K);
    }
}

}  // namespace culsh
