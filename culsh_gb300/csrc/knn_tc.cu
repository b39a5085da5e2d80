// Candidate distances and top-K on the 5th-generation tensor cores for
// queries whose candidate sets cover a large share of the dataset.
//
// Replaces, for such queries, the host collect/sort/unique of
// cuLSH_SearchTables.cu:321-364, the distance kernel of
// cuLSH_Kernels.cu:301-348 (launched by cuLSH_Querying.cu:284-343) and the
// top-K of cuLSH_Kernels.cu:356-456. Results are those of the exact FP32
// path: the same ids and bit-identical squared distances.
//
// Formulation. A query's candidates are marked in an N-bit membership row
// (k_cand_bitmap, candidates.cu). A tile of 128 queries is multiplied with
// every 256- (or 128-) point tile of the dataset by tcgen05.mma
// (q . x in FP32 accumulators in TMEM, bf16 operands staged by TMA), and the
// epilogue turns each accumulator into a ranking key
//     t = w_x - 2 q.x,     w_x = |x|^2 (exact form) or |x|^2 - C S_x (bound form)
// so that d = t + |q|^2 (exact form) or t + |q|^2 - C S_q <= d (bound form).
// Each query keeps the Kl smallest keys among its candidates (membership
// bit set) in shared memory; a chunk of 32 columns is only examined when its
// smallest key beats the query's current Kl-th key.
//
//  * Exact form: every coordinate of the dataset and the queries is an
//    integer with |v| <= 256 (exact in bf16), and D max|v|^2 < 2^24 and
//    D (max v - min v)^2 < 2^24. Every product, partial sum and norm is then an
//    integer below 2^24, so the tensor-core sum is exact in any order, t is
//    exact, and d = t + |q|^2 is the exact squared distance, which is also
//    what the reference's FP32 lane order computes (all of its partial sums
//    are exact too). One bf16 product per element.
//  * Bound form (any finite data): q = qh + ql, x = xh + xl split into bf16
//    parts; the tensor cores sum qh.xh + qh.xl + ql.xh. With S = |q|^2 + |x|^2
//    (upper bounds), |d~ - d| <= C S covers the split residue, the
//    accumulation, the norms and the FP32 lane order of the exact distance,
//    so key + base is a lower bound of the exact distance. The merge kernel
//    recomputes the exact FP32 lane-order distance of the listed candidates
//    in ascending bound order and stops once the bound passes the K-th exact
//    distance. A query whose full list's largest bound does not exceed its
//    K-th exact distance (the list was too short to prove the result) is
//    re-run by the exact per-query kernel.
//
// Work split: the (query tile, point tile) pairs are cut into gridDim.x
// contiguous ranges, one per persistent CTA, so that every CTA does the same
// number of tensor-core tiles. A CTA's range covers part of one or a few
// query tiles; for each it leaves one partial list per query (list set
// blockIdx.x + query tile, unique because the ranges are ordered), which the
// merge kernel combines.
//
// Roles: warp 0 issues TMA loads (the query tile's operand once per query
// tile, point tiles into a ring, membership words and per-point weights into
// a second ring); warp 1 owns TMEM and issues tcgen05.mma (M = 128, N = the
// point tile, K = 16 per instruction) into two accumulators, so that the
// epilogue of one tile overlaps the products of the next; the other warps read
// TMEM with tcgen05.ld and keep the per-query lists. Every mbarrier wait is
// bounded: on timeout the kernel raises kErrSpin, drains its copies and
// products, frees TMEM and returns; the host then reports the error.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "culsh_internal.cuh"
#include "topk_common.cuh"

namespace culsh {
namespace {

constexpr int KM = 128;                 // rows of one MMA (TMEM lanes)
// Tile shapes: MQ queries (MQ / 128 MMAs of M = 128) x BN points per tile,
// NEPI epilogue warps, NCH = 32 NEPI / MQ column slices of 64 per query.
constexpr int kBnExact = 128, kMqExact = 256, kNepiExact = 16;   // exact form: two MMAs share a point tile
constexpr int kBnBound = 128, kMqBound = 128, kNepiBound = 8;    // bound form: three products per element
constexpr int kNchExact = 32 * kNepiExact / kMqExact, kNchBound = 32 * kNepiBound / kMqBound;
// Bounded waits: each poll suspends the thread in hardware for up to
// kKnnSuspendNs (it resumes as soon as the phase completes, and takes no issue
// slots meanwhile), at most kKnnPoll polls (a few seconds) in all.
constexpr uint32_t kKnnPoll = 1u << 18;
constexpr uint32_t kKnnSuspendNs = 16384;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool bar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity), "r"(kKnnSuspendNs)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase of the given parity; on timeout raises the
// block's abort flag and kErrSpin.
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, int* err) {
    for (uint32_t i = 0; i < kKnnPoll; ++i) {
        if (bar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
    }
    *abort_flag = 1;
    atomicOr(err, kErrSpin);
    return false;
}
// Bounded wait that ignores the abort flag (draining at exit).
__device__ __forceinline__ void bar_drain(uint64_t* bar, uint32_t parity, int* err) {
    for (uint32_t i = 0; i < kKnnPoll; ++i)
        if (bar_try_wait(bar, parity)) return;
    atomicOr(err, kErrSpin);
}

__device__ __forceinline__ void tma_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_addr(bar)), "r"(x), "r"(y)
        : "memory");
}
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// K-major operand, 128-byte swizzle, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(
            d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// The 32 accumulator columns [taddr, taddr + 32) of this thread's TMEM lane,
// loaded and waited for in one statement, so that no use of r can be
// scheduled before the wait.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
}

// Element k (0..31) of 32 register values, by a tree of selects on k's bits
// (no local memory).
__device__ __forceinline__ float select32(const uint32_t* v, int k) {
    float a[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) a[i] = __uint_as_float((k & 1) ? v[2 * i + 1] : v[2 * i]);
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = (k & 2) ? a[2 * i + 1] : a[2 * i];
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = (k & 4) ? a[2 * i + 1] : a[2 * i];
#pragma unroll
    for (int i = 0; i < 2; ++i) a[i] = (k & 8) ? a[2 * i + 1] : a[2 * i];
    return (k & 16) ? a[1] : a[0];
}

// Three-input minimum (sm_100 and later).
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Order-preserving encoding of a float key as an unsigned word (unsigned
// comparison of encodings = float comparison of keys), so that a shared bound
// can be lowered with atomicMin.
__host__ __device__ __forceinline__ uint32_t key_enc(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_dec(uint32_t e) {
    return __uint_as_float((e & 0x80000000u) ? (e & 0x7FFFFFFFu) : ~e);
}
constexpr uint32_t kNoBound = 0xFF800000u;   // key_enc(+infinity)

// Exact form of the search (see the file comment), from the flags and value
// ranges of the dataset and of the dense queries.
__device__ __forceinline__ bool exact_form(const KnnState* ds, const KnnState* qs, int D) {
    if ((ds->flags | qs->flags) & (kKnnNotSmallInt | kKnnNonFinite)) return false;
    const int mneg = max(ds->mneg, qs->mneg), mpos = max(ds->mpos, qs->mpos);
    if (mneg == 0 || mpos == 0) return false;
    const long long lo = 257 - mneg, hi = mpos - 257;
    const long long mag = max(-lo, hi);
    return (long long)D * mag * mag < (1ll << 24) && (long long)D * (hi - lo) * (hi - lo) < (1ll << 24);
}

struct KnnArgs {
    int N, D, Dp;
    int exact_launched;               // the exact form's kernel is part of this search
    long long ntp_exact, ntp_bound;   // point tiles of 256 / 128
    int kl_exact, kl_bound;
    int op_stages, ep_stages;
    const unsigned int* n_dense;
    const KnnState* dstate;
    const KnnState* qstate;
    unsigned int* qbound;             // [dense position] shared key bound of the exact form (key_enc)
    const float* w_exact;
    const float* w_bound;
    float* part_key;
    uint32_t* part_id;
    int* part_n;
    int* err;
};

// The CTA whose range of (query tile, point tile) pairs holds pair p: ranges
// are [c U / G, (c + 1) U / G).
__device__ __forceinline__ int owner_cta(long long p, long long U, int G) {
    return (int)(((p + 1) * G - 1) / U);
}

// MQ queries per tile (MQ / 128 MMAs of M = 128 share each point tile of BN
// points), NEPI epilogue warps: each lane keeps one query's list over one of
// the NCH column slices of the tile (32 * NEPI == MQ * NCH).
template <int BN, int MQ, int NEPI, bool kExact>
__global__ void __launch_bounds__(64 + 32 * NEPI, 1)
    k_knn_tc(const __grid_constant__ CUtensorMap tm_qh, const __grid_constant__ CUtensorMap tm_ql,
             const __grid_constant__ CUtensorMap tm_xh, const __grid_constant__ CUtensorMap tm_xl,
             const __grid_constant__ CUtensorMap tm_bm, KnnArgs a) {
    constexpr int NT = 32 * NEPI;          // list-keeping threads: one (query, column slice) each
    constexpr int MH = MQ / KM;            // M = 128 halves of the query tile
    constexpr int NCH = NT / MQ;           // column slices of a tile
    constexpr int CW = BN / NCH;           // columns per slice
    constexpr int BW = BN / 32;            // membership words per query row and point tile
    constexpr uint32_t kTmemCols = 2 * MH * BN;
    static_assert(NCH * MQ == NT && CW == 64, "64-column slices, one list per (query, slice)");
    // the other form's kernel runs (the exact one only where it was launched)
    if ((a.exact_launched && exact_form(a.dstate, a.qstate, a.D)) != kExact) return;
    const unsigned int nd = *a.n_dense;
    const long long nqt = ((long long)nd + MQ - 1) / MQ;
    const long long ntp = kExact ? a.ntp_exact : a.ntp_bound;
    const long long U = nqt * ntp;
    const int G = (int)min((long long)gridDim.x, U);
    if ((int)blockIdx.x >= G) return;
    const long long p0 = (long long)blockIdx.x * U / G, p1 = (long long)(blockIdx.x + 1) * U / G;
    const int Dp = a.Dp, atoms = Dp / 64, ksteps = Dp / 16;
    const int Kl = kExact ? a.kl_exact : a.kl_bound;
    const int ops = a.op_stages, eps = a.ep_stages;
    const int need_xl = kExact ? 0 : ((a.dstate->flags & kKnnHasLo) != 0);
    const int need_ql = kExact ? 0 : ((a.qstate->flags & kKnnHasLo) != 0);

    extern __shared__ __align__(1024) unsigned char smraw[];
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
    const uint32_t qbytes = (uint32_t)MQ * Dp * 2, xbytes = (uint32_t)BN * Dp * 2;
    unsigned char* sQh = base;
    unsigned char* sQl = sQh + qbytes;                                  // bound form only
    unsigned char* sX = sQh + (kExact ? 1u : 2u) * qbytes;             // op ring: [xh][xl] per stage
    const uint32_t op_stride = (kExact ? 1u : 2u) * xbytes;
    unsigned char* sE = sX + (size_t)ops * op_stride;                  // ep ring: [membership][weights] per stage
    const uint32_t bm_bytes = (uint32_t)MQ * BW * 4, w_bytes = (uint32_t)BN * 4;
    const uint32_t ep_stride = bm_bytes + w_bytes;
    float* lkey = reinterpret_cast<float*>(sE + (size_t)eps * ep_stride);   // [Kl][NT]
    uint32_t* lid = reinterpret_cast<uint32_t*>(lkey + (size_t)Kl * NT);
    uint64_t* bars = reinterpret_cast<uint64_t*>(lid + (size_t)Kl * NT);
    uint64_t* a_full = bars;
    uint64_t* a_empty = bars + 1;
    uint64_t* tfull = bars + 2;     // [2]
    uint64_t* tempty = bars + 4;    // [2]
    uint64_t* done_bar = bars + 6;
    uint64_t* full_op = bars + 7;             // [ops]
    uint64_t* empty_op = full_op + ops;       // [ops]
    uint64_t* full_ep = empty_op + ops;       // [eps]
    uint64_t* empty_ep = full_ep + eps;       // [eps]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(empty_ep + eps);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        bar_init(a_full, 1);
        bar_init(a_empty, 1);
        for (int s = 0; s < 2; ++s) {
            bar_init(tfull + s, 1);
            bar_init(tempty + s, NEPI);
        }
        bar_init(done_bar, 1);
        for (int s = 0; s < ops; ++s) {
            bar_init(full_op + s, 1);
            bar_init(empty_op + s, 1);
        }
        for (int s = 0; s < eps; ++s) {
            bar_init(full_ep + s, 1);
            bar_init(empty_ep + s, NEPI);
        }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // ---- TMA producer ----
        long long cur_qt = -1;
        int j = -1;
        long long i = 0;
        // (query tile, point tile) of pair p and both rings' stage and round
        // parity, advanced incrementally (no 64-bit division per tile)
        long long qt = p0 / ntp, pt = p0 - qt * ntp;
        int s = 0, e = 0;
        uint32_t spar = 0, epar = 0;
        long long issued_op = 0, issued_ep = 0;   // copies issued into each ring
        for (long long p = p0; p < p1 && !*abort_flag; ++p, ++i) {
            if (qt != cur_qt) {
                ++j;
                cur_qt = qt;
                if (j >= 1 && !bar_wait(a_empty, (uint32_t)((j - 1) & 1), abort_flag, a.err)) break;
                bar_expect_tx(a_full, qbytes * (need_ql ? 2u : 1u));
                for (int k = 0; k < atoms; ++k) {
                    tma_2d(sQh + (size_t)k * MQ * 128, &tm_qh, a_full, k * 64, (int)(qt * MQ));
                    if (need_ql) tma_2d(sQl + (size_t)k * MQ * 128, &tm_ql, a_full, k * 64, (int)(qt * MQ));
                }
            }
            if (i >= ops && !bar_wait(empty_op + s, spar ^ 1u, abort_flag, a.err)) break;
            unsigned char* xs = sX + (size_t)s * op_stride;
            bar_expect_tx(full_op + s, xbytes * (need_xl ? 2u : 1u));
            for (int k = 0; k < atoms; ++k) {
                tma_2d(xs + (size_t)k * BN * 128, &tm_xh, full_op + s, k * 64, (int)(pt * BN));
                if (need_xl) tma_2d(xs + xbytes + (size_t)k * BN * 128, &tm_xl, full_op + s, k * 64, (int)(pt * BN));
            }
            ++issued_op;
            if (i >= eps && !bar_wait(empty_ep + e, epar ^ 1u, abort_flag, a.err)) break;
            unsigned char* es = sE + (size_t)e * ep_stride;
            bar_expect_tx(full_ep + e, ep_stride);
            tma_2d(es, &tm_bm, full_ep + e, (int)(pt * BW), (int)(qt * MQ));
            bulk_copy(es + bm_bytes, (kExact ? a.w_exact : a.w_bound) + pt * BN, w_bytes, full_ep + e);
            ++issued_ep;
            if (++s == ops) { s = 0; spar ^= 1u; }
            if (++e == eps) { e = 0; epar ^= 1u; }
            if (++pt == ntp) { pt = 0; ++qt; }
        }
        // Drain: every copy issued into a ring stage completes before exit.
        for (int st = 0; st < ops && st < issued_op; ++st) {
            const long long last = st + ((issued_op - 1 - st) / ops) * ops;
            bar_drain(full_op + st, (uint32_t)((last / ops) & 1), a.err);
        }
        for (int et = 0; et < eps && et < issued_ep; ++et) {
            const long long last = et + ((issued_ep - 1 - et) / eps) * eps;
            bar_drain(full_ep + et, (uint32_t)((last / eps) & 1), a.err);
        }
        if (j >= 0) bar_drain(a_full, (uint32_t)(j & 1), a.err);
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        // kind::f16: FP32 accumulator, bf16 A and B, both K-major, N = BN, M = 128.
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                               ((uint32_t)(KM >> 4) << 24);
        const uint64_t qhdesc = desc_sw128(smem_addr(sQh)), qldesc = desc_sw128(smem_addr(sQl));
        const uint64_t xdesc = desc_sw128(smem_addr(sX));
        long long cur_qt = -1;
        int j = -1;
        long long i = 0;
        long long qt = p0 / ntp, pt = p0 - qt * ntp;
        int s = 0;
        uint32_t spar = 0;
        for (long long p = p0; p < p1; ++p, ++i) {
            if (qt != cur_qt) {
                if (j >= 0) mma_commit(a_empty);
                ++j;
                cur_qt = qt;
                if (!bar_wait(a_full, (uint32_t)(j & 1), abort_flag, a.err)) break;
            }
            if (++pt == ntp) { pt = 0; ++qt; }
            const int acc = (int)(i & 1);
            if (i >= 2 && !bar_wait(tempty + acc, (uint32_t)(((i >> 1) - 1) & 1), abort_flag, a.err)) break;
            if (!bar_wait(full_op + s, spar, abort_flag, a.err)) break;
            fence_after();
            // descriptors advance by adding the byte offset / 16 to their
            // start-address field (shared addresses stay below 2^18: no carry)
            const uint64_t dxh = xdesc + (uint64_t)(s * (op_stride >> 4)), dxl = dxh + (xbytes >> 4);
            for (int hq = 0; hq < MH; ++hq) {
                const uint32_t d = tmem + (uint32_t)((acc * MH + hq) * BN);
#pragma unroll 4
                for (int ks = 0; ks < ksteps; ++ks) {
                    const uint64_t ao = (uint64_t)(((ks >> 2) * MQ * 128 + hq * KM * 128 + (ks & 3) * 32) >> 4);
                    const uint64_t bo = (uint64_t)(((ks >> 2) * BN * 128 + (ks & 3) * 32) >> 4);
                    mma_bf16(d, qhdesc + ao, dxh + bo, idesc, ks > 0 ? 1u : 0u);
                    if (!kExact) {
                        if (need_xl) mma_bf16(d, qhdesc + ao, dxl + bo, idesc, 1u);
                        if (need_ql) mma_bf16(d, qldesc + ao, dxh + bo, idesc, 1u);
                    }
                }
            }
            mma_commit(empty_op + s);
            mma_commit(tfull + acc);
            if (++s == ops) { s = 0; spar ^= 1u; }
        }
        // every product has landed before TMEM is released
        mma_commit(done_bar);
        bar_drain(done_bar, 0, a.err);
    } else if (warp >= 2) {
        // ---- epilogue: ranking keys, per-query lists ----
        const int ew = warp - 2;
        const int quad = warp & 3;                    // TMEM lanes this warp may read
        const int hq = (ew >> 2) % MH;                // query half (its own accumulator)
        const int ch = (ew >> 2) / MH;                // column slice
        const int row = hq * KM + quad * 32 + lane;   // query of the tile
        const int lt = ew * 32 + lane;
        float* mk = lkey + lt;
        uint32_t* mi = lid + lt;
        int n = 0;
        float thr = INFINITY;
        long long cur_qt = -1;
        long long i = 0;
        // Exact form: the lists of one query (column slices, CTAs) share a
        // bound in global memory, the smallest K-th key of any full list (an
        // upper bound of the query's K-th key: that list holds K candidates at
        // or below it). A candidate above it cannot be in the top-K; one equal
        // to it still enters (it may win the tie on its id).
        auto flush = [&](long long qt) {
            const long long lst = ((long long)blockIdx.x + qt) * NCH + ch;
            const long long lb = lst * (long long)Kl;
            for (int k = 0; k < n; ++k) {
                a.part_key[(lb + k) * MQ + row] = mk[k * NT];
                a.part_id[(lb + k) * MQ + row] = mi[k * NT];
            }
            a.part_n[lst * MQ + row] = n;
        };
        long long qt = p0 / ntp, pt = p0 - qt * ntp;
        int e = 0;
        uint32_t epar = 0;
        for (long long p = p0; p < p1; ++p, ++i) {
            if (qt != cur_qt) {
                if (cur_qt >= 0) flush(cur_qt);
                cur_qt = qt;
                n = 0;
                thr = INFINITY;
            }
            const int acc = (int)(i & 1);
            const int gq = (int)qt * MQ + row;   // dense position of this lane's query
            // the shared bound is read before the waits (its latency overlaps
            // them): it only decreases, so an earlier value is still a bound
            const uint32_t ext_enc = kExact ? __ldcg(a.qbound + gq) : 0u;
            // every lane waits (and so sees the copied data); the warp leaves
            // together if any lane gave up, since tcgen05.ld is warp-wide
            const bool ok = bar_wait(tfull + acc, (uint32_t)((i >> 1) & 1), abort_flag, a.err) &&
                            bar_wait(full_ep + e, epar, abort_flag, a.err);
            if (!__all_sync(0xffffffffu, ok)) break;
            fence_after();
            const unsigned char* es = sE + (size_t)e * ep_stride;
            const float ext = kExact ? key_dec(ext_enc) : INFINITY;
            // a key enters iff key < thr and key <= ext, i.e. key < lim
            const float ext_up = nextafterf(ext, INFINITY);
            float lim = fminf(thr, ext_up);
            const uint2 mw = *reinterpret_cast<const uint2*>(es + (size_t)row * BW * 4 + ch * 8);   // 2 words: 64 columns
            const float* wv = reinterpret_cast<const float*>(es + bm_bytes) + ch * CW;
            const uint32_t id0 = (uint32_t)(pt * BN + ch * CW);
            const uint32_t tbase =
                tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)((acc * MH + hq) * BN + ch * CW);
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                // The slice's two 32-column halves are loaded and ranked in
                // turn, so that only 32 keys are live at a time; the
                // accumulator goes back to the MMA warp as soon as the second
                // half is in registers (the next products into it overlap the
                // rest of this tile's key work).
                uint32_t rc[32];
                if (c == 1) __syncwarp();   // tcgen05.ld is warp-collective: reconverge after the inserts
                tmem_ld32(tbase + (uint32_t)(c * 32), rc);
                if (c == 1) {
                    fence_before();
                    __syncwarp();
                    if (lane == 0) bar_arrive(tempty + acc);
                }
                // keys t = w - 2 q.x (packed FMA, in place)
#pragma unroll
                for (int j = 0; j < 32; j += 4) {
                    const float4 w4 = *reinterpret_cast<const float4*>(wv + c * 32 + j);
                    const float2 a2 = __ffma2_rn(make_float2(-2.0f, -2.0f),
                                                 make_float2(__uint_as_float(rc[j]), __uint_as_float(rc[j + 1])),
                                                 make_float2(w4.x, w4.y));
                    const float2 b2 = __ffma2_rn(make_float2(-2.0f, -2.0f),
                                                 make_float2(__uint_as_float(rc[j + 2]), __uint_as_float(rc[j + 3])),
                                                 make_float2(w4.z, w4.w));
                    rc[j] = __float_as_uint(a2.x);
                    rc[j + 1] = __float_as_uint(a2.y);
                    rc[j + 2] = __float_as_uint(b2.x);
                    rc[j + 3] = __float_as_uint(b2.y);
                }
                const uint32_t mbits = c == 0 ? mw.x : mw.y;
                float mm[11];
#pragma unroll
                for (int k = 0; k < 10; ++k)
                    mm[k] = fmin3(__uint_as_float(rc[3 * k]), __uint_as_float(rc[3 * k + 1]), __uint_as_float(rc[3 * k + 2]));
                mm[10] = fminf(__uint_as_float(rc[30]), __uint_as_float(rc[31]));
                const float m = fmin3(fmin3(mm[0], mm[1], mm[2]), fmin3(mm[3], mm[4], mm[5]),
                                      fmin3(fmin3(mm[6], mm[7], mm[8]), mm[9], mm[10]));
                if (m < lim && mbits) {
                    // this lane's candidate columns whose key beats its list;
                    // lanes insert in parallel, each into its own sorted list
                    uint32_t pm = 0;
#pragma unroll
                    for (int k = 0; k < 32; ++k) pm |= (__uint_as_float(rc[k]) < lim ? 1u : 0u) << k;
                    pm &= mbits;
                    for (; pm; pm &= pm - 1) {
                        const int k = __ffs((int)pm) - 1;
                        const float key = select32(rc, k);
                        if (!(key < lim)) continue;
                        // ids arrive in ascending order, so a key equal to a
                        // listed one goes after it
                        int pos = n < Kl ? n : Kl - 1;
                        while (pos > 0 && mk[(pos - 1) * NT] > key) {
                            mk[pos * NT] = mk[(pos - 1) * NT];
                            mi[pos * NT] = mi[(pos - 1) * NT];
                            --pos;
                        }
                        mk[pos * NT] = key;
                        mi[pos * NT] = id0 + (uint32_t)(c * 32 + k);
                        if (n < Kl) ++n;
                        if (n == Kl) {
                            thr = mk[(Kl - 1) * NT];
                            lim = fminf(thr, ext_up);
                        }
                    }
                }
            }
            if (kExact && n == Kl && thr < ext) atomicMin(a.qbound + gq, key_enc(thr));
            __syncwarp();
            if (lane == 0) bar_arrive(empty_ep + e);
            if (++e == eps) { e = 0; epar ^= 1u; }
            if (++pt == ntp) { pt = 0; ++qt; }
        }
        if (cur_qt >= 0 && !*abort_flag) flush(cur_qt);
    }
    __syncthreads();
    fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}


// bf16 parts, squared norm and bound weight of rows (the dataset once per
// index, the dense queries once per search), and the rows' flags. Row r is
// src[list ? list[r] : r]; there are *count rows (or n). Rows from there up to
// the padded count (a multiple of pad_to, or pad) are zero rows with weight
// FLT_MAX. sq[r] = |x|^2 (RN FP32 chain, exact for small integers);
// wb[r] = |x|^2 - C |x|^2_up rounded down (the bound form's weight, and for a
// query its base). One warp per row.
__global__ void k_knn_rows(const float* __restrict__ src, int D, int Dp, const int* __restrict__ list,
                           const unsigned int* __restrict__ count, int64_t n, int64_t pad, int pad_to,
                           __nv_bfloat16* __restrict__ xh, __nv_bfloat16* __restrict__ xl, float* __restrict__ sq,
                           float* __restrict__ wb, float C, KnnState* __restrict__ st,
                           unsigned int* __restrict__ bound) {
    const int lane = threadIdx.x & 31;
    const int64_t nrows = count ? (int64_t)*count : n;
    const int64_t npad = count ? ((nrows + pad_to - 1) / pad_to) * pad_to : pad;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    int flags = 0, mneg = 0, mpos = 0;
    for (int64_t r = w0; r < npad; r += nw) {
        if (bound && lane == 0) bound[r] = kNoBound;
        if (r >= nrows) {
            if (r < n || count) {   // operand rows exist only up to the buffer's rows
                for (int d = lane; d < Dp; d += 32) {
                    xh[r * Dp + d] = __float2bfloat16_rn(0.0f);
                    xl[r * Dp + d] = __float2bfloat16_rn(0.0f);
                }
            }
            if (lane == 0) {
                sq[r] = FLT_MAX;
                wb[r] = FLT_MAX;
            }
            continue;
        }
        const float* row = src + (list ? (int64_t)list[r] : r) * D;
        float s = 0.0f, su = 0.0f;
        for (int d = lane; d < Dp; d += 32) {
            const float x = d < D ? __ldg(row + d) : 0.0f;
            const __nv_bfloat16 h = __float2bfloat16_rn(x);
            const __nv_bfloat16 l = __float2bfloat16_rn(__fsub_rn(x, __bfloat162float(h)));
            xh[r * Dp + d] = h;
            xl[r * Dp + d] = l;
            if (__bfloat16_as_ushort(l) & 0x7FFF) flags |= kKnnHasLo;
            if (!(fabsf(x) <= FLT_MAX)) flags |= kKnnNonFinite;
            if (x == rintf(x) && fabsf(x) <= 256.0f) {
                const int v = (int)x;
                mneg = max(mneg, 257 - v);
                mpos = max(mpos, v + 257);
            } else {
                flags |= kKnnNotSmallInt;
            }
            s = __fmaf_rn(x, x, s);
            su = __fmaf_ru(x, x, su);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s = __fadd_rn(s, __shfl_xor_sync(0xffffffffu, s, o));
            su = __fadd_ru(su, __shfl_xor_sync(0xffffffffu, su, o));
        }
        if (lane == 0) {
            sq[r] = s;
            wb[r] = __fsub_rd(s, __fmul_ru(C, su));
        }
    }
    const unsigned full = 0xffffffffu;
    flags = __reduce_or_sync(full, flags);
    mneg = __reduce_max_sync(full, mneg);
    mpos = __reduce_max_sync(full, mpos);
    if (lane == 0) {
        if (flags) atomicOr(&st->flags, flags);
        if (mneg) atomicMax(&st->mneg, mneg);
        if (mpos) atomicMax(&st->mpos, mpos);
    }
}

// Exact FP32 squared distance in the reference's lane order
// (cuLSH_Kernels.cu:323-346): partial j chains columns j, j+8, ... with FMA,
// then (p0+p4, p1+p5, p2+p6, p3+p7) -> (t0+t2) + (t1+t3). One thread.
__device__ __forceinline__ float lane_order_distance(const float* __restrict__ q, const float* __restrict__ x, int D) {
    float p[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) p[j] = 0.0f;
    int c = 0;
    for (; c + 8 <= D; c += 8) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const float df = __fsub_rn(__ldg(q + c + j), __ldg(x + c + j));
            p[j] = __fmaf_rn(df, df, p[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (c + j < D) {
            const float df = __fsub_rn(__ldg(q + c + j), __ldg(x + c + j));
            p[j] = __fmaf_rn(df, df, p[j]);
        }
    const float t0 = __fadd_rn(p[0], p[4]), t1 = __fadd_rn(p[1], p[5]);
    const float t2 = __fadd_rn(p[2], p[6]), t3 = __fadd_rn(p[3], p[7]);
    return __fadd_rn(__fadd_rn(t0, t2), __fadd_rn(t1, t3));
}

constexpr int MERGE_WARPS = 4;
constexpr int kEpStages = 4;   // membership / weight ring stages

// Merges the partial lists of each dense query into its top-K (one warp per
// query). Lists are walked in ascending key order and left as soon as the
// lower bound key + base passes the K-th distance found so far. Exact form:
// key + |q|^2 is the distance. Bound form: the exact FP32 lane-order distance
// of each entry not yet excluded is recomputed; a query with a full list whose
// last bound does not exceed its K-th distance is handed to the fallback list.
__global__ void __launch_bounds__(32 * MERGE_WARPS) k_knn_merge(KnnSearch k) {
    __shared__ float s_d[MERGE_WARPS][kMaxKnnK];
    __shared__ uint32_t s_i[MERGE_WARPS][kMaxKnnK];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned int nd = *k.n_dense;
    const bool exact = k.exact_possible && exact_form(k.dstate, k.qstate, k.D);
    const int K = k.K;
    const int Kl = exact ? k.kl_exact : k.kl_bound;
    const int MQ = exact ? kMqExact : kMqBound;
    const int NCH = exact ? kNchExact : kNchBound;
    const int BN = exact ? kBnExact : kBnBound;
    const long long ntp = (k.N + BN - 1) / BN;
    const long long nqt = ((long long)nd + MQ - 1) / MQ;
    const long long U = nqt * ntp;
    const int G = (int)min((long long)k.grid, U);
    float* wd = s_d[w];
    uint32_t* wi = s_i[w];
    for (long long i = (long long)blockIdx.x * MERGE_WARPS + w; i < nd; i += (long long)gridDim.x * MERGE_WARPS) {
        const int q = k.dense_q[i];
        const long long qt = i / MQ;
        const int r = (int)(i - qt * MQ);
        const int c0 = owner_cta(qt * ntp, U, G), c1 = owner_cta(qt * ntp + ntp - 1, U, G);
        const float base = exact ? k.qsq[i] : k.qbase[i];
        const float* qrow = k.queries + (int64_t)q * k.D;
        int n = 0;
        float thr_d = FLT_MAX;
        uint32_t thr_i = 0;
        float minlast = INFINITY;   // smallest last bound over the full lists
        for (int c = c0; c <= c1; ++c) {
            for (int h = 0; h < NCH; ++h) {   // the column slices
                const long long lst = ((long long)c + qt) * NCH + h;
                const int cnt = k.part_n[lst * MQ + r];
                const long long lb = lst * (long long)Kl;
                if (!exact && cnt == Kl)
                    minlast = fminf(minlast, __fadd_rd(k.part_key[(lb + Kl - 1) * MQ + r], base));
                for (int e0 = 0; e0 < cnt; e0 += 32) {
                    const int e = e0 + lane;
                    const bool valid = e < cnt;
                    const float key = valid ? k.part_key[(lb + e) * MQ + r] : INFINITY;
                    const uint32_t id = valid ? k.part_id[(lb + e) * MQ + r] : 0u;
                    const float low = exact ? __fadd_rn(key, base) : __fadd_rd(key, base);
                    // entries are in ascending key order: lane 0 holds the chunk's smallest
                    if (__shfl_sync(0xffffffffu, low, 0) > thr_d) break;
                    float d = INFINITY;
                    if (valid && low <= thr_d) d = exact ? low : lane_order_distance(qrow, k.X + (int64_t)id * k.D, k.D);
                    uint32_t want = __ballot_sync(0xffffffffu, valid && lessp(d, id, thr_d, thr_i));
                    while (want) {
                        const int src = __ffs(want) - 1;
                        want &= want - 1;
                        const float cd = __shfl_sync(0xffffffffu, d, src);
                        const uint32_t cid = __shfl_sync(0xffffffffu, id, src);
                        if (lessp(cd, cid, thr_d, thr_i)) warp_insert(wd, wi, n, K, cd, cid, thr_d, thr_i);
                    }
                }
            }
        }
        if (!exact && minlast <= thr_d) {
            // a list may have dropped an entry that belongs to the top-K
            if (lane == 0) k.fallback[atomicAdd(k.n_fallback, 1u)] = q;
            continue;
        }
        int32_t* oid = k.out_ids + (int64_t)q * K;
        float* od = k.out_d + (int64_t)q * K;
        for (int j = lane; j < K; j += 32) {
            oid[j] = j < n ? (int32_t)wi[j] : -1;
            od[j] = j < n ? wd[j] : FLT_MAX;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// host side

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn knn_encode_fn() {
    static std::atomic<EncodeTiledFn> fn{nullptr};
    EncodeTiledFn f = fn.load();
    if (!f) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f = reinterpret_cast<EncodeTiledFn>(p);
        fn = f;
    }
    return f;
}

// 2-D map over a row-major [rows][cols] array with a (box_cols x box_rows) box.
bool knn_map(CUtensorMap* m, const void* ptr, CUtensorMapDataType dt, int esize, uint64_t cols, uint64_t rows,
             uint32_t box_cols, uint32_t box_rows, bool swizzle) {
    EncodeTiledFn fn = knn_encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * (uint64_t)esize};
    const cuuint32_t box[2] = {box_cols, box_rows};
    const cuuint32_t es[2] = {1, 1};
    return fn(m, dt, 2, const_cast<void*>(ptr), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
              swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t knn_smem(bool exact, int Dp, int Kl, int ops, int eps) {
    const int MQ = exact ? kMqExact : kMqBound, BN = exact ? kBnExact : kBnBound;
    const int nepi = exact ? kNepiExact : kNepiBound;
    const size_t q = (size_t)MQ * Dp * 2 * (exact ? 1 : 2);
    const size_t op = (size_t)BN * Dp * 2 * (exact ? 1 : 2);
    const size_t ep = (size_t)MQ * (BN / 32) * 4 + (size_t)BN * 4;
    const size_t lists = (size_t)32 * nepi * Kl * 8;   // one list per (query, column slice)
    const size_t bars = 8 * (7 + 2 * ops + 2 * eps) + 16;
    return 1024 + q + ops * op + eps * ep + lists + bars;
}

template <int BN, int MQ, int NEPI, bool kExact>
cudaError_t launch_knn_form(const KnnSearch& k, const CUtensorMap& mxh, const CUtensorMap& mxl, cudaStream_t s) {
    static std::atomic<size_t> cap{0};
    const size_t smem = kExact ? k.smem_exact : k.smem_bound;
    if (smem > cap.load()) {
        const cudaError_t e = cudaFuncSetAttribute(k_knn_tc<BN, MQ, NEPI, kExact>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        cap = smem;
    }
    CUtensorMap mbm, mqh, mql;
    if (!knn_map(&mbm, k.bm, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, (uint64_t)k.nwp, (uint64_t)k.Qcap, BN / 32, MQ,
                 false) ||
        !knn_map(&mqh, k.qh, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (uint64_t)k.Dp, (uint64_t)k.Qcap, 64, MQ, true) ||
        !knn_map(&mql, k.ql, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (uint64_t)k.Dp, (uint64_t)k.Qcap, 64, MQ, true))
        return cudaErrorNotSupported;
    KnnArgs a;
    a.N = k.N;
    a.D = k.D;
    a.Dp = k.Dp;
    a.exact_launched = k.exact_possible;
    a.ntp_exact = (k.N + kBnExact - 1) / kBnExact;
    a.ntp_bound = (k.N + kBnBound - 1) / kBnBound;
    a.kl_exact = k.kl_exact;
    a.kl_bound = k.kl_bound;
    a.op_stages = kExact ? k.ops_exact : k.ops_bound;
    a.ep_stages = kEpStages;
    a.n_dense = k.n_dense;
    a.dstate = k.dstate;
    a.qstate = k.qstate;
    a.qbound = k.qbound;
    a.w_exact = k.w_exact;
    a.w_bound = k.w_bound;
    a.part_key = k.part_key;
    a.part_id = k.part_id;
    a.part_n = k.part_n;
    a.err = k.err;
    k_knn_tc<BN, MQ, NEPI, kExact><<<k.grid, 64 + 32 * NEPI, smem, s>>>(mqh, mql, mxh, mxl, mbm, a);
    return cudaGetLastError();
}

}  // namespace

float knn_bound_factor(int D) {
    // split residue (three products) and accumulation of 3D products, as in
    // the projection's bound; the exact distance's own FP32 lane order
    // (gamma_n, n = ceil(D/8) + 6, twice: d~ <= 2 S); norms and key
    // arithmetic ((D + 16) u); all with a 10 % margin.
    const double u = std::ldexp(1.0, -24), u23 = std::ldexp(1.0, -23), u16 = std::ldexp(1.0, -16);
    const double kappa = 1.25 * (3.02 * u16 + (3.0 * D + 16) * u23);
    const double nn = (double)((D + 7) / 8 + 6);
    const double gamma = nn * u / (1.0 - nn * u);
    return std::nextafter((float)(1.1 * (kappa + 2.0 * gamma + (D + 16) * u)), INFINITY);
}

bool knn_plan(KnnSearch& k, int max_smem) {
    if (k.D < 1 || k.D > 128 || k.K < 1 || k.K > kMaxKnnK || k.N < 1) return false;
    k.Dp = (k.D + 63) / 64 * 64;
    k.kl_exact = k.K;
    // bound form: K plus a margin of entries that the error bound may reorder;
    // CULSH_KNN_LIST_MARGIN sets the margin (the tests use 0 to reach the
    // exact fallback)
    int margin = std::max(8, k.K / 2);
    if (const char* e = getenv("CULSH_KNN_LIST_MARGIN")) margin = std::max(0, atoi(e));
    k.kl_bound = std::min(kMaxKnnK, k.K + margin);
    k.ops_exact = k.ops_bound = 0;
    // the deepest point-tile ring (1 to 4 stages) that fits
    for (int ops = 4; ops >= 1 && !k.ops_exact; --ops) {
        const size_t sm = knn_smem(true, k.Dp, k.kl_exact, ops, kEpStages);
        if (sm <= (size_t)max_smem) {
            k.ops_exact = ops;
            k.smem_exact = sm;
        }
    }
    for (int ops = 4; ops >= 1 && !k.ops_bound; --ops) {
        const size_t sm = knn_smem(false, k.Dp, k.kl_bound, ops, kEpStages);
        if (sm <= (size_t)max_smem) {
            k.ops_bound = ops;
            k.smem_bound = sm;
        }
    }
    // the bound form serves every search; the exact form only when it fits too
    if (!k.ops_bound) return false;
    if (!k.ops_exact) k.exact_possible = 0;
    k.nwp = (int)((((int64_t)k.N + 31) / 32 + 3) / 4 * 4);
    return true;
}

size_t knn_part_lists(const KnnSearch& k) {
    // list sets blockIdx.x + query tile < grid + Qcap / MQ, with MQ rows and
    // NCH column slices each
    const size_t e = (size_t)(k.grid + k.Qcap / kMqExact) * kMqExact * kNchExact;
    const size_t b = (size_t)(k.grid + k.Qcap / kMqBound) * kMqBound * kNchBound;
    return std::max(e, b);
}
size_t knn_part_entries(const KnnSearch& k) {
    return knn_part_lists(k) * (size_t)std::max(k.kl_exact, k.kl_bound);
}

cudaError_t launch_knn_rows_dataset(const float* X, int64_t N, int D, int Dp, void* xh, void* xl, float* w_exact,
                                    float* w_bound, int64_t pad, float C, KnnState* st, cudaStream_t s) {
    const int blocks = (int)std::min<int64_t>((pad * 32 + 255) / 256, 152 * 16);
    k_knn_rows<<<blocks, 256, 0, s>>>(X, D, Dp, nullptr, nullptr, N, pad, 1, static_cast<__nv_bfloat16*>(xh),
                                      static_cast<__nv_bfloat16*>(xl), w_exact, w_bound, C, st, nullptr);
    return cudaGetLastError();
}

int knn_launches(const KnnSearch& k) { return 3 + (k.exact_possible ? 1 : 0); }

cudaError_t launch_knn_search(const KnnSearch& k, cudaStream_t s) {
    // query rows in dense-list order, zero rows up to the next tile
    const int qblocks = (int)std::min<int64_t>(((int64_t)k.Qcap * 32 + 255) / 256, 152 * 8);
    k_knn_rows<<<qblocks, 256, 0, s>>>(k.queries, k.D, k.Dp, k.dense_q, k.n_dense, 0, 0, std::max(kMqExact, kMqBound),
                                       static_cast<__nv_bfloat16*>(k.qh), static_cast<__nv_bfloat16*>(k.ql), k.qsq,
                                       k.qbase, k.C, k.qstate, k.qbound);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (k.exact_possible) {
        CUtensorMap mxh;
        if (!knn_map(&mxh, k.xh, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (uint64_t)k.Dp, (uint64_t)k.N, 64, kBnExact,
                     true))
            return cudaErrorNotSupported;
        e = launch_knn_form<kBnExact, kMqExact, kNepiExact, true>(k, mxh, mxh, s);
        if (e != cudaSuccess) return e;
    }
    CUtensorMap mxh, mxl;
    if (!knn_map(&mxh, k.xh, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (uint64_t)k.Dp, (uint64_t)k.N, 64, kBnBound, true) ||
        !knn_map(&mxl, k.xl, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (uint64_t)k.Dp, (uint64_t)k.N, 64, kBnBound, true))
        return cudaErrorNotSupported;
    e = launch_knn_form<kBnBound, kMqBound, kNepiBound, false>(k, mxh, mxl, s);
    if (e != cudaSuccess) return e;
    const int mblocks = (int)std::min<int64_t>(((int64_t)k.Qcap + MERGE_WARPS - 1) / MERGE_WARPS, 152 * 16);
    k_knn_merge<<<mblocks, 32 * MERGE_WARPS, 0, s>>>(k);
    return cudaGetLastError();
}

}  // namespace culsh
