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

}  // namespace culsh
