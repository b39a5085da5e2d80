// K1 on the 5th-generation tensor cores (tcgen05 + TMA + TMEM).
//
// Replaces, for index builds, the per-table cublasSgemm + -b + /W + floor of
// cuLSH_Indexing.cu:27-66 and cuLSH_Kernels.cu:40-101 with one persistent
// GEMM over all L*M columns whose epilogue produces the exact canonical FP32
// bucket codes.
//
// Exactness. X = Xh + Xl and A = Ah + Al are split into bf16 parts (Xl is
// skipped when the data are exactly representable in bf16). The tensor cores
// compute y = Xh*Ah' + Xh*Al' (+ Xl*Ah') with FP32 accumulation in TMEM.
// For each element the distance between y and the canonical sequential FMA
// chain is bounded by E = kappa * |x|_2 * |a|_2 (Cauchy-Schwarz on sum|x||a|),
// where kappa covers the split residue (2^-16 per omitted cross term), a
// rounding at every accumulation of the tensor-core sum (one 2^-23 step per
// product) and the canonical chain's own rounding ((D + 2) * 2^-24), with a
// 1.25 margin. A cheap window test on (y - b) * (1/W) proves most codes
// without the two IEEE divides. Because fl(fl(t - b) / W)
// is non-decreasing in t, floor(v(y - E)) == floor(v(y + E)) proves the code;
// every other element is appended to a list and recomputed in the canonical
// order by k_tc_recompute. Codes are therefore bit-identical to the SIMT
// kernel and the oracle.
//
// Structure: persistent CTAs of 18 warps. Warp 0 issues TMA loads (the
// projection matrix once, then 128-point X tiles into a 1- or 2-stage ring);
// warp 1 owns TMEM and issues tcgen05.mma (M=128, N=L*M padded to 16, K=16
// per instruction, bf16 inputs, FP32 accumulators, two accumulators so that
// the epilogue of one tile overlaps the MMAs of the next); warps 2-17 read
// TMEM with tcgen05.ld (four warps per lane quadrant, each taking a quarter
// of the columns) and run the epilogue. Codes the bound leaves open are appended
// row by row to a per-CTA list. Every mbarrier wait is bounded:
// on timeout the kernel raises kErrSpin and the host falls back to the SIMT
// kernel.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cfloat>
#include <climits>

#include "culsh_internal.cuh"

namespace culsh {
namespace {

constexpr int TC_M = 128;
constexpr int TC_EPI_WARPS = 16;                      // four per TMEM lane quadrant
constexpr int TC_THREADS = 64 + 32 * TC_EPI_WARPS;    // TMA warp, MMA warp, epilogue
constexpr uint32_t kPollLimit = 1u << 26;

struct TcArgs {
    int64_t N;
    int D, Dp, LM, LMp, ntiles, need_lo, stages, tmem_cols;
    float W, kappa;
    const float* b;        // [LM]
    const float* anorm;    // [LM] upper bounds of |a_c|_2
    const float* xnorm;    // [N]  upper bounds of |x_n|_2
    int32_t* codes;        // [LM][N]
    int32_t* pmin;         // [gridDim.x][LM]
    int32_t* pmax;
    unsigned long long* relist;   // (n << 16) | c of codes to recompute, one region per CTA
    unsigned long long relist_cap;        // entries per CTA region
    unsigned int* relist_cnt;             // [gridDim.x] entries used per region (may exceed the cap)
    float inv_w;                          // 1/W rounded to nearest
    int* err;
    uint32_t b_bytes, x_bytes;    // one bf16 operand region of A (LMp x Dp) / of an X tile (128 x Dp)
    // Streaming form (A too large to keep in shared memory): this launch
    // covers columns [col0, col0 + LM) of LMtot; each ring stage holds one
    // 64-wide K slice of Xh (Xl) and of Ah, Al.
    int col0, LMtot;
    uint32_t stage_bytes;         // streaming: bytes of one ring stage
    uint32_t a_chunk;             // streaming: bytes of one A slice (LMp x 64 bf16)
    int list_continue;            // streaming: recompute lists continue from relist_cnt
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the completion of the phase with the given parity. The
// single-thread producer and MMA roles back off between polls so that their
// spinning does not take issue slots from the epilogue warps.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, int* err,
                                          bool backoff = false) {
    for (uint32_t i = 0; i < kPollLimit; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
        if (backoff) __nanosleep(64);
    }
    *abort_flag = 1;
    atomicOr(err, kErrSpin);
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// groups 1024 bytes apart (stride byte offset), sm_100 descriptor version.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(
            d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// kStream = false: A resident in shared memory (Dp, LMp <= 256), X tiles
// ring-buffered. kStream = true: X and A both streamed in 64-wide K slices,
// for any Dp; a launch covers at most 256 columns. Same epilogue.
template <bool kStream>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_project_tc(const __grid_constant__ CUtensorMap tm_xh, const __grid_constant__ CUtensorMap tm_xl,
                 const __grid_constant__ CUtensorMap tm_ah, const __grid_constant__ CUtensorMap tm_al, TcArgs a) {
    extern __shared__ __align__(1024) unsigned char smraw[];
    // 1024-byte aligned operand regions (the swizzle atoms assume it).
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
    unsigned char* sAh = base;
    unsigned char* sAl = sAh + (kStream ? 0 : a.b_bytes);
    // resident: stage s = Xh at s*(1+need_lo)*x_bytes, Xl right after;
    // streaming: stage s = [Xh slice][Xl slice][Ah slice][Al slice]
    unsigned char* sX = kStream ? base : sAl + a.b_bytes;
    const uint32_t stage_bytes = kStream ? a.stage_bytes : a.x_bytes * (a.need_lo ? 2u : 1u);
    unsigned char* tail = sX + (size_t)a.stages * stage_bytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(tail);
    uint64_t* empty = full + 2;
    uint64_t* tfull = empty + 2;
    uint64_t* tempty = tfull + 2;
    uint64_t* bfull = tempty + 2;
    uint32_t* tmem_ptr = reinterpret_cast<uint32_t*>(bfull + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_ptr + 1);
    unsigned int* list_top = reinterpret_cast<unsigned int*>(tmem_ptr + 2);
    int32_t* cmin = reinterpret_cast<int32_t*>(tmem_ptr + 4);
    int32_t* cmax = cmin + a.LMp;
    float* s_an = reinterpret_cast<float*>(cmax + a.LMp);     // |a_c|_2 bounds
    float* s_b = s_an + a.LMp;                                 // b_c
    uint32_t* s_unsure = reinterpret_cast<uint32_t*>(s_b + a.LMp);   // [8 words][TC_EPI_WARPS * 32] per-thread masks

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
            mbar_init(tfull + s, 1);
            mbar_init(tempty + s, TC_EPI_WARPS);
        }
        mbar_init(bfull, 1);
        *abort_flag = 0;
        *list_top = a.list_continue ? a.relist_cnt[blockIdx.x] : 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int c = tid; c < a.LMp; c += TC_THREADS) {
        cmin[c] = INT_MAX;
        cmax[c] = INT_MIN;
        s_an[c] = c < a.LM ? __ldg(a.anorm + a.col0 + c) : 0.0f;
        s_b[c] = c < a.LM ? __ldg(a.b + a.col0 + c) : 0.0f;
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_ptr)),
                     "r"((uint32_t)a.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_ptr;
    const int katoms = a.Dp / 64, ksteps = a.Dp / 16;

    if (kStream && warp == 0 && lane == 0) {
        // ---- TMA producer, streaming: every tile, every K slice of X and A ----
        const uint32_t xb = 16384u;   // one X slice: 128 rows x 128 bytes
        int i = 0;
        for (int tile = blockIdx.x; tile < a.ntiles && !*abort_flag; tile += gridDim.x) {
            for (int k = 0; k < katoms; ++k, ++i) {
                const int s = i % a.stages;
                if (i >= a.stages &&
                    !mbar_wait(empty + s, (uint32_t)((i / a.stages - 1) & 1), abort_flag, a.err, true))
                    break;
                unsigned char* st = sX + (size_t)s * stage_bytes;
                unsigned char* sa = st + xb * (a.need_lo ? 2u : 1u);
                mbar_expect_tx(full + s, stage_bytes);
                tma_load_2d(st, &tm_xh, full + s, k * 64, tile * TC_M);
                if (a.need_lo) tma_load_2d(st + xb, &tm_xl, full + s, k * 64, tile * TC_M);
                tma_load_2d(sa, &tm_ah, full + s, k * 64, a.col0);
                tma_load_2d(sa + a.a_chunk, &tm_al, full + s, k * 64, a.col0);
            }
        }
    } else if (kStream && warp == 1 && lane == 0) {
        // ---- MMA issuer, streaming ----
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(a.LMp >> 3) << 17) |
                               ((uint32_t)(TC_M >> 4) << 24);
        const uint32_t xb = 16384u;
        int i = 0, t = 0;
        bool ok = true;
        for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += gridDim.x, ++t) {
            const int acc = t & 1;
            if (t >= 2 && !mbar_wait(tempty + acc, (uint32_t)(((t >> 1) - 1) & 1), abort_flag, a.err, true)) break;
            const uint32_t d = tmem + (uint32_t)(acc * a.LMp);
            for (int k = 0; k < katoms; ++k, ++i) {
                const int s = i % a.stages;
                if (!mbar_wait(full + s, (uint32_t)((i / a.stages) & 1), abort_flag, a.err, true)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t xh = smem_u32(sX + (size_t)s * stage_bytes);
                const uint32_t ah = xh + xb * (a.need_lo ? 2u : 1u), al = ah + a.a_chunk;
                for (int ks = 0; ks < 4; ++ks) {
                    const uint32_t o = (uint32_t)(ks * 32);
                    umma_bf16(d, sw128_desc(xh + o), sw128_desc(ah + o), idesc, (k > 0 || ks > 0) ? 1u : 0u);
                    umma_bf16(d, sw128_desc(xh + o), sw128_desc(al + o), idesc, 1u);
                    if (a.need_lo) umma_bf16(d, sw128_desc(xh + xb + o), sw128_desc(ah + o), idesc, 1u);
                }
                umma_commit(empty + s);
            }
            if (!ok) break;
            umma_commit(tfull + acc);
        }
    } else if (!kStream && warp == 0 && lane == 0) {
        // ---- TMA producer ----
        mbar_expect_tx(bfull, 2 * a.b_bytes);
        for (int k = 0; k < katoms; ++k) {
            tma_load_2d(sAh + (size_t)k * a.LMp * 128, &tm_ah, bfull, k * 64, 0);
            tma_load_2d(sAl + (size_t)k * a.LMp * 128, &tm_al, bfull, k * 64, 0);
        }
        int i = 0;
        for (int tile = blockIdx.x; tile < a.ntiles && !*abort_flag; tile += gridDim.x, ++i) {
            const int s = i % a.stages;
            if (i >= a.stages && !mbar_wait(empty + s, (uint32_t)((i / a.stages - 1) & 1), abort_flag, a.err, true))
                break;
            unsigned char* xh = sX + (size_t)s * stage_bytes;
            mbar_expect_tx(full + s, stage_bytes);
            for (int k = 0; k < katoms; ++k) {
                tma_load_2d(xh + (size_t)k * TC_M * 128, &tm_xh, full + s, k * 64, tile * TC_M);
                if (a.need_lo) tma_load_2d(xh + a.x_bytes + (size_t)k * TC_M * 128, &tm_xl, full + s, k * 64, tile * TC_M);
            }
        }
    } else if (!kStream && warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        // kind::f16 instruction descriptor: FP32 accumulator, bf16 A and B,
        // both K-major, N = LMp, M = 128.
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(a.LMp >> 3) << 17) |
                               ((uint32_t)(TC_M >> 4) << 24);
        if (mbar_wait(bfull, 0, abort_flag, a.err, true)) {
            int i = 0;
            for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x, ++i) {
                const int s = i % a.stages, acc = i & 1;
                if (i >= 2 && !mbar_wait(tempty + acc, (uint32_t)(((i >> 1) - 1) & 1), abort_flag, a.err, true)) break;
                if (!mbar_wait(full + s, (uint32_t)((i / a.stages) & 1), abort_flag, a.err, true)) break;
                tc_fence_after();
                const uint32_t d = tmem + (uint32_t)(acc * a.LMp);
                const uint32_t xh = smem_u32(sX + (size_t)s * stage_bytes);
                const uint32_t ah = smem_u32(sAh), al = smem_u32(sAl);
                for (int ks = 0; ks < ksteps; ++ks) {
                    const uint32_t xo = (uint32_t)((ks >> 2) * TC_M * 128 + (ks & 3) * 32);
                    const uint32_t bo = (uint32_t)((ks >> 2) * a.LMp * 128 + (ks & 3) * 32);
                    umma_bf16(d, sw128_desc(xh + xo), sw128_desc(ah + bo), idesc, ks > 0 ? 1u : 0u);
                    umma_bf16(d, sw128_desc(xh + xo), sw128_desc(al + bo), idesc, 1u);
                    if (a.need_lo) umma_bf16(d, sw128_desc(xh + a.x_bytes + xo), sw128_desc(ah + bo), idesc, 1u);
                }
                umma_commit(empty + s);
                umma_commit(tfull + acc);
            }
        }
    } else if (warp >= 2) {
        // ---- epilogue: TMEM -> proven codes, list of codes to recompute ----
        const int ew = warp - 2;
        const int quad = warp & 3;                 // TMEM lane quadrant this warp may access
        const int part = ew >> 2;                  // which quarter of the column chunks
        const int row = quad * 32 + lane;
        const int nchunk = a.LMp / 16;
        const int ch0 = part * nchunk / 4, ch1 = (part + 1) * nchunk / 4;
        uint32_t* my_mask = s_unsure + ew * 32 + lane;   // word w at my_mask[w * TC_EPI_WARPS * 32]
        unsigned long long* region = a.relist + (unsigned long long)blockIdx.x * a.relist_cap;
        int i = 0;
        for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x, ++i) {
            const int acc = i & 1;
            if (!mbar_wait(tfull + acc, (uint32_t)((i >> 1) & 1), abort_flag, a.err)) break;
            tc_fence_after();
            const int64_t n = (int64_t)tile * TC_M + row;
            const bool valid = n < a.N;
            const float kx = __fmul_ru(a.kappa, valid ? __ldg(a.xnorm + n) : 0.0f);
            uint32_t nuns = 0;
            for (int ch = ch0; ch < ch1; ++ch) {
                const int c0 = ch * 16;
                uint32_t r[16];
                tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(acc * a.LMp + c0), r);
                int32_t* out = a.codes + (int64_t)(a.col0 + c0) * a.N + n;
                uint32_t unsure = 0;
                int32_t mylo = INT_MAX, myhi = INT_MIN;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int c = c0 + j;
                    const float y = __uint_as_float(r[j]);
                    const float E = __fmul_ru(kx, s_an[c]);
                    const float bc = s_b[c];
                    // Cheap rigorous test first: v_approx is within |v| * 2^-21 +
                    // 2^-40 of the canonical v of any t in [y - E, y + E] widened
                    // by E/W; no integer in that window proves the code.
                    const float va = (y - bc) * a.inv_w;
                    const float fa = floorf(va);
                    const float win = __fmul_ru(E, a.inv_w) * 1.0001f + fabsf(va) * 4.8e-7f + 1e-12f;
                    bool sure = va - fa > win && (fa + 1.0f) - va > win && fabsf(va) < 2.0e9f;
                    float fl = fa;
                    if (!sure) {
                        fl = floorf(__fdiv_rn(__fsub_rn(__fsub_rd(y, E), bc), a.W));
                        const float fh = floorf(__fdiv_rn(__fsub_rn(__fadd_ru(y, E), bc), a.W));
                        sure = fl == fh && fl >= -2147483648.0f && fl < 2147483648.0f;
                    }
                    const bool live = valid && c < a.LM;
                    const int32_t code = sure ? (int32_t)fl : 0;
                    if (live) out[(int64_t)j * a.N] = code;
                    if (live && !sure) unsure |= 1u << j;
                    const bool use = live && sure;
                    const int32_t lo = __reduce_min_sync(0xffffffffu, use ? code : INT_MAX);
                    const int32_t hi = __reduce_max_sync(0xffffffffu, use ? code : INT_MIN);
                    if (lane == j) {
                        mylo = lo;
                        myhi = hi;
                    }
                }
                if (lane < 16 && mylo <= myhi) {
                    atomicMin(cmin + c0 + lane, mylo);
                    atomicMax(cmax + c0 + lane, myhi);
                }
                // bit (ch - ch0) * 16 + j of this thread's mask words
                const int w = (ch - ch0) >> 1;
                const uint32_t bits = unsure << (((ch - ch0) & 1) * 16);
                if (((ch - ch0) & 1) == 0) my_mask[w * TC_EPI_WARPS * 32] = bits;
                else my_mask[w * TC_EPI_WARPS * 32] |= bits;
                nuns += __popc(unsure);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(tempty + acc);
            // Append this row's unsure columns contiguously (one atomic per warp).
            uint32_t incl = nuns;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
            if (total) {
                unsigned int basei = 0;
                if (lane == 31) basei = atomicAdd(list_top, total);
                basei = __shfl_sync(0xffffffffu, basei, 31);
                unsigned long long pos = (unsigned long long)basei + incl - nuns;
                const int nwords = (ch1 - ch0 + 1) >> 1;
                for (int w = 0; w < nwords && nuns; ++w) {
                    for (uint32_t m = my_mask[w * TC_EPI_WARPS * 32]; m; m &= m - 1) {
                        const int c = a.col0 + ch0 * 16 + w * 32 + (__ffs(m) - 1);
                        if (pos < a.relist_cap) region[pos] = ((unsigned long long)n << 16) | (unsigned)c;
                        ++pos;
                    }
                }
            }
        }
    }
    __syncthreads();
    for (int c = tid; c < a.LM; c += TC_THREADS) {
        a.pmin[(int64_t)blockIdx.x * a.LMtot + a.col0 + c] = cmin[c];
        a.pmax[(int64_t)blockIdx.x * a.LMtot + a.col0 + c] = cmax[c];
    }
    if (tid == 0) a.relist_cnt[blockIdx.x] = *list_top;
    tc_fence_after();
    if (warp == 1) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)a.tmem_cols)
                     : "memory");
    }
}

// Splits X into bf16 parts and bounds the row norms from above (warp per row).
__global__ void k_split_rows(const float* __restrict__ X, int64_t N, int D, int Dp, __nv_bfloat16* __restrict__ xh,
                             __nv_bfloat16* __restrict__ xl, float* __restrict__ xnorm, int* __restrict__ flags) {
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    int any_lo = 0, bad = 0;
    for (int64_t n = w0; n < N; n += nw) {
        const float* row = X + n * D;
        float ss = 0.0f;
        for (int d = lane; d < Dp; d += 32) {
            const float x = d < D ? __ldg(row + d) : 0.0f;
            const __nv_bfloat16 h = __float2bfloat16_rn(x);
            const __nv_bfloat16 l = __float2bfloat16_rn(__fsub_rn(x, __bfloat162float(h)));
            xh[n * Dp + d] = h;
            xl[n * Dp + d] = l;
            any_lo |= __bfloat16_as_ushort(l) & 0x7FFF;
            bad |= !(fabsf(x) <= FLT_MAX);
            ss = __fmaf_ru(x, x, ss);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ss = __fadd_ru(ss, __shfl_xor_sync(0xffffffffu, ss, o));
        if (lane == 0) xnorm[n] = __fmul_ru(__fsqrt_ru(ss), 1.0009765625f);
    }
    if (__any_sync(0xffffffffu, any_lo != 0) && lane == 0) atomicOr(flags, 1);
    if (__any_sync(0xffffffffu, bad != 0) && lane == 0) atomicOr(flags, 2);
}

// Canonical-order recomputation of the codes the tensor-core bound could not
// prove (one thread per list entry; entries of CTA region r are
// list[r * cap .. r * cap + cnt[r])).
__global__ void k_tc_recompute(const float* __restrict__ X, int64_t N, int D, const float* __restrict__ A,
                               const float* __restrict__ b, float W, const unsigned long long* __restrict__ list,
                               unsigned long long cap, const unsigned int* __restrict__ cnt, int regions, int LM,
                               int stage_a, int32_t* __restrict__ codes, int32_t* __restrict__ cmin,
                               int32_t* __restrict__ cmax, int* __restrict__ err) {
    // A staged in shared memory with padded rows, so that the lanes of a warp
    // (different columns, same d) hit different banks: D + 4 floats when
    // D % 4 == 0 (16-byte reads; column c starts at bank 4c mod 32), else D + 1.
    extern __shared__ __align__(16) float sA[];
    __shared__ int32_t smin[1024], smax[1024];   // per-column ranges of this block (LM <= 1024 here)
    const int Dq = (D & 3) == 0 ? D + 4 : D + 1;
    const bool block_range = LM <= 1024;
    if (block_range)
        for (int c = threadIdx.x; c < LM; c += blockDim.x) {
            smin[c] = INT_MAX;
            smax[c] = INT_MIN;
        }
    if (stage_a)
        for (int i = threadIdx.x; i < LM * D; i += blockDim.x) sA[(i / D) * Dq + (i % D)] = __ldg(A + i);
    __syncthreads();
    // Blocks walk the regions (region r is list[r * cap .. r * cap + cnt[r])).
    for (int r = blockIdx.x % regions, part = blockIdx.x / regions, parts = (gridDim.x + regions - 1) / regions;
         r < regions; r += gridDim.x) {
      const unsigned int nr = min((unsigned long long)__ldg(cnt + r), cap);
      for (unsigned int k = part * blockDim.x + threadIdx.x; k < nr; k += parts * blockDim.x) {
        const unsigned long long e = list[(unsigned long long)r * cap + k];
        const int64_t n = (int64_t)(e >> 16);
        const int c = (int)(e & 0xFFFF);
        const float* x = X + n * D;
        float acc = 0.0f;
        if (stage_a && (D & 3) == 0) {
            const float* av = sA + (int64_t)c * Dq;
            for (int d = 0; d < D; d += 4) {
                const float4 x4 = __ldg(reinterpret_cast<const float4*>(x + d));
                const float4 a4 = *reinterpret_cast<const float4*>(av + d);
                acc = __fmaf_rn(x4.x, a4.x, acc);
                acc = __fmaf_rn(x4.y, a4.y, acc);
                acc = __fmaf_rn(x4.z, a4.z, acc);
                acc = __fmaf_rn(x4.w, a4.w, acc);
            }
        } else if (stage_a) {
            const float* av = sA + (int64_t)c * Dq;
            for (int d = 0; d < D; ++d) acc = __fmaf_rn(__ldg(x + d), av[d], acc);
        } else if ((D & 3) == 0) {
            // A too large for shared memory (high D): 16-byte loads of the
            // row and of the column's A row from L2, same FMA order
            const float* av = A + (int64_t)c * D;
#pragma unroll 4
            for (int d = 0; d < D; d += 4) {
                const float4 x4 = __ldg(reinterpret_cast<const float4*>(x + d));
                const float4 a4 = __ldg(reinterpret_cast<const float4*>(av + d));
                acc = __fmaf_rn(x4.x, a4.x, acc);
                acc = __fmaf_rn(x4.y, a4.y, acc);
                acc = __fmaf_rn(x4.z, a4.z, acc);
                acc = __fmaf_rn(x4.w, a4.w, acc);
            }
        } else {
            const float* av = A + (int64_t)c * D;
            for (int d = 0; d < D; ++d) acc = __fmaf_rn(__ldg(x + d), __ldg(av + d), acc);
        }
        const float v = __fdiv_rn(__fsub_rn(acc, __ldg(b + c)), W);
        const float f = floorf(v);
        int32_t code = 0;
        if (!(fabsf(f) <= FLT_MAX)) atomicOr(err, kErrNonFinite);
        else if (!(f >= -2147483648.0f && f < 2147483648.0f)) atomicOr(err, kErrCodeRange);
        else code = (int32_t)f;
        codes[(int64_t)c * N + n] = code;
        if (block_range) {
            atomicMin(smin + c, code);
            atomicMax(smax + c, code);
        } else {
            atomicMin(cmin + c, code);
            atomicMax(cmax + c, code);
        }
      }
    }
    if (block_range) {
        __syncthreads();
        for (int c = threadIdx.x; c < LM; c += blockDim.x) {
            if (smin[c] <= smax[c]) {
                atomicMin(cmin + c, smin[c]);
                atomicMax(cmax + c, smax[c]);
            }
        }
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

bool make_map(CUtensorMap* m, const void* ptr, uint64_t cols, uint64_t rows, uint32_t box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 2};
    const cuuint32_t box[2] = {64, box_rows};
    const cuuint32_t es[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

TcPlan tc_plan(int64_t N, int D, int LM, int num_sms, int max_smem) {
    TcPlan p{};
    p.Dp = (D + 63) / 64 * 64;
    p.LMp = (LM + 15) / 16 * 16;
    p.ok = N >= 1024 && p.Dp <= 256 && p.LMp >= 16 && p.LMp <= 256 && LM <= 65535 && N < (1ll << 47);
    if (!p.ok) return p;
    p.b_bytes = (uint32_t)p.LMp * p.Dp * 2;
    p.x_bytes = (uint32_t)TC_M * p.Dp * 2;
    // operands, barriers, per-column ranges / norms / offsets, per-thread masks
    const size_t fixed = 1024 + 2 * (size_t)p.b_bytes + 128 + 16 * (size_t)p.LMp + 8 * 4 * TC_EPI_WARPS * 32;
    int tc = 32;
    while (tc < 2 * p.LMp) tc <<= 1;
    p.tmem_cols = tc;
    p.ntiles = (int)((N + TC_M - 1) / TC_M);
    p.grid = std::min(p.ntiles, num_sms);
    for (int need_lo = 0; need_lo < 2; ++need_lo) {
        const size_t st = (size_t)p.x_bytes * (need_lo ? 2 : 1);
        int stages = 2;
        while (stages > 0 && fixed + stages * st > (size_t)max_smem) --stages;
        p.stages[need_lo] = stages;
        p.smem[need_lo] = fixed + stages * st;
    }
    p.ok = p.stages[1] >= 1;
    return p;
}

cudaError_t launch_split_rows(const float* X, int64_t N, int D, int Dp, void* xh, void* xl, float* xnorm, int* flags,
                              cudaStream_t st) {
    const int blocks = (int)std::min<int64_t>((N * 32 + 255) / 256, 152 * 16);
    k_split_rows<<<blocks, 256, 0, st>>>(X, N, D, Dp, static_cast<__nv_bfloat16*>(xh),
                                        static_cast<__nv_bfloat16*>(xl), xnorm, flags);
    return cudaGetLastError();
}

cudaError_t launch_project_tc(const TcPlan& p, int need_lo, int64_t N, int D, int LM, const void* xh, const void* xl,
                              const void* ah, const void* al, const float* b, const float* anorm, const float* xnorm,
                              float W, float kappa, int32_t* codes, int32_t* pmin, int32_t* pmax,
                              unsigned long long* relist, unsigned long long relist_cap, unsigned int* relist_cnt,
                              int* err, cudaStream_t st) {
    CUtensorMap mxh, mxl, mah, mal;
    if (!make_map(&mxh, xh, p.Dp, N, TC_M) || !make_map(&mxl, xl, p.Dp, N, TC_M) ||
        !make_map(&mah, ah, p.Dp, p.LMp, p.LMp) || !make_map(&mal, al, p.Dp, p.LMp, p.LMp))
        return cudaErrorNotSupported;
    TcArgs a;
    a.N = N;
    a.D = D;
    a.Dp = p.Dp;
    a.LM = LM;
    a.LMp = p.LMp;
    a.ntiles = p.ntiles;
    a.need_lo = need_lo;
    a.stages = p.stages[need_lo];
    a.tmem_cols = p.tmem_cols;
    a.W = W;
    a.kappa = kappa;
    a.b = b;
    a.anorm = anorm;
    a.xnorm = xnorm;
    a.codes = codes;
    a.pmin = pmin;
    a.pmax = pmax;
    a.relist = relist;
    a.relist_cap = relist_cap;
    a.relist_cnt = relist_cnt;
    a.inv_w = 1.0f / W;
    a.err = err;
    a.b_bytes = p.b_bytes;
    a.x_bytes = p.x_bytes;
    a.col0 = 0;
    a.LMtot = LM;
    a.stage_bytes = 0;
    a.a_chunk = 0;
    a.list_continue = 0;
    const int smem = (int)p.smem[need_lo];
    cudaError_t e = cudaFuncSetAttribute(k_project_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_project_tc<false><<<p.grid, TC_THREADS, smem, st>>>(mxh, mxl, mah, mal, a);
    return cudaGetLastError();
}

TcStreamPlan tc_plan_stream(int64_t N, int D, int LM, int num_sms, int max_smem) {
    TcStreamPlan p{};
    p.Dp = (D + 63) / 64 * 64;
    p.LMp = (LM + 15) / 16 * 16;
    p.ok = N >= 1024 && p.Dp <= 16384 && LM <= 65535 && N < (1ll << 47);
    if (!p.ok) return p;
    p.ntiles = (int)((N + TC_M - 1) / TC_M);
    p.grid = std::min(p.ntiles, num_sms);
    p.ok = false;
    for (int need_lo = 0; need_lo < 2; ++need_lo) {
        // widest column block whose two-stage (or one-stage) ring fits
        for (int blk = 256; blk >= 16; blk -= 16) {
            const size_t stage = 16384u * (need_lo ? 2u : 1u) + 2u * (size_t)blk * 128u;
            const size_t tail = 128 + 16 * (size_t)blk + 8 * 4 * TC_EPI_WARPS * 32;
            int stages = 2;
            while (stages > 0 && 1024 + stages * stage + tail > (size_t)max_smem) --stages;
            if (stages == 0) continue;
            p.blk[need_lo] = std::min(blk, p.LMp);
            p.stages[need_lo] = stages;
            p.smem[need_lo] = 1024 + stages * (16384u * (need_lo ? 2u : 1u) + 2u * (size_t)p.blk[need_lo] * 128u) +
                              128 + 16 * (size_t)p.blk[need_lo] + 8 * 4 * TC_EPI_WARPS * 32;
            break;
        }
    }
    p.ok = p.stages[1] >= 1 && p.stages[0] >= 1;
    return p;
}

cudaError_t launch_project_tc_stream(const TcStreamPlan& p, int need_lo, int64_t N, int D, int LM, const void* xh,
                                     const void* xl, const void* ah, const void* al, const float* b,
                                     const float* anorm, const float* xnorm, float W, float kappa, int32_t* codes,
                                     int32_t* pmin, int32_t* pmax, unsigned long long* relist,
                                     unsigned long long relist_cap, unsigned int* relist_cnt, int* err,
                                     cudaStream_t st) {
    const int blk = p.blk[need_lo];
    CUtensorMap mxh, mxl;
    if (!make_map(&mxh, xh, p.Dp, N, TC_M) || !make_map(&mxl, xl, p.Dp, N, TC_M)) return cudaErrorNotSupported;
    const int smem = (int)p.smem[need_lo];
    cudaError_t e = cudaFuncSetAttribute(k_project_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(relist_cnt, 0, sizeof(unsigned int) * (size_t)p.grid, st);
    if (e != cudaSuccess) return e;
    for (int col0 = 0; col0 < LM; col0 += blk) {
        const int lmc = std::min(blk, LM - col0);      // columns of this launch
        const int lmp = (lmc + 15) / 16 * 16;           // padded to the MMA's N granularity
        CUtensorMap mah, mal;
        if (!make_map(&mah, ah, p.Dp, (uint64_t)p.LMp, (uint32_t)lmp) ||
            !make_map(&mal, al, p.Dp, (uint64_t)p.LMp, (uint32_t)lmp))
            return cudaErrorNotSupported;
        TcArgs a;
        a.N = N;
        a.D = D;
        a.Dp = p.Dp;
        a.LM = lmc;
        a.LMp = lmp;
        a.ntiles = p.ntiles;
        a.need_lo = need_lo;
        a.stages = p.stages[need_lo];
        int tc = 32;
        while (tc < 2 * lmp) tc <<= 1;
        a.tmem_cols = tc;
        a.W = W;
        a.kappa = kappa;
        a.b = b;
        a.anorm = anorm;
        a.xnorm = xnorm;
        a.codes = codes;
        a.pmin = pmin;
        a.pmax = pmax;
        a.relist = relist;
        a.relist_cap = relist_cap;
        a.relist_cnt = relist_cnt;
        a.inv_w = 1.0f / W;
        a.err = err;
        a.b_bytes = 0;
        a.x_bytes = 16384u;
        a.col0 = col0;
        a.LMtot = LM;
        a.a_chunk = (uint32_t)lmp * 128u;
        a.stage_bytes = 16384u * (need_lo ? 2u : 1u) + 2u * a.a_chunk;
        a.list_continue = 1;
        k_project_tc<true><<<p.grid, TC_THREADS, smem, st>>>(mxh, mxl, mah, mal, a);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_tc_recompute(const float* X, int64_t N, int D, int LM, const float* A, const float* b, float W,
                                const unsigned long long* list, unsigned long long cap, const unsigned int* cnt,
                                int regions, int32_t* codes, int32_t* cmin, int32_t* cmax, int* err, cudaStream_t st) {
    const size_t smem = sizeof(float) * (size_t)LM * ((D & 3) == 0 ? D + 4 : D + 1);
    const int stage_a = smem <= 200 * 1024;
    if (stage_a) {
        cudaError_t e = cudaFuncSetAttribute(k_tc_recompute, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    // Grid: a multiple of the region count, so that every block has a region.
    // 512 threads: with A staged (up to ~100 KB at L*M = 192, D = 128) two
    // blocks fit an SM, 32 warps to cover the latency of the X row loads.
    const int grid = regions * (stage_a ? 2 : 8);
    k_tc_recompute<<<grid, 512, stage_a ? smem : 0, st>>>(
        X, N, D, A, b, W, list, cap, cnt, regions, LM, stage_a, codes, cmin, cmax, err);
    return cudaGetLastError();
}

}  // namespace culsh
