// K1: projection of points onto all L*M stacked LSH columns with the
// bucket-code epilogue fused in.
//
// Replaces cuLSH_Indexing.cu:27-66 (cublasSgemm + kernel_subtractVectorFromMatrixRows
// + kernel_divideMatrixWithScalar) and cuLSH_Kernels.cu:91-101 (kernel_floorMatrix),
// which the reference runs once per table with a full dataset upload each time.
// Here one launch covers every table: C[n][c] = sum_d X[n][d] * A[c][d] over
// c = l*M + m, then v = fl(fl(C) - b) / W and code = floor(v).
//
// Arithmetic is the canonical FP32 order: each output is one fused
// multiply-add chain over d = 0..D-1 in ascending order (register-tiled, the
// tiling never reorders a chain), so codes are bit-exact against the CPU
// oracle. The FP32 FMA pipe bounds this kernel (2*N*D*L*M flops).
#include <algorithm>
#include <cfloat>
#include <climits>

#include "culsh_internal.cuh"

namespace culsh {
namespace {

constexpr int NT = 256;   // threads: 16 (points) x 16 (columns), each PT x CT outputs

// Block tile BN = 16*PT points x BC = 16*CT columns, BK dimensions per
// shared-memory stage. Index builds use PT = 8, CT = 4, BK = 16; query batches
// take one of five tilings the search tuner picks (PT x CT = 4x8 by default,
// 2x8, 8x4, 4x4, 2x4: fewer shared-memory loads per FMA against more blocks
// in flight), and 2x12 (all of L*M <= 192 columns in one block) when the
// queries are read straight from host memory and copied to the device on
// the way (xcopy).
//
// Thread (tx, ty) owns points 32*(i/2) + 2*tx + (i%2), i < PT, so that a
// half-warp's float2 reads of the X tile cover 128 contiguous bytes (no bank
// conflicts), and columns ty*CT .. ty*CT+CT-1. The projection matrix is read
// transposed (AT[d][c], rows of lmp >= LM floats, columns past LM zero) with
// coalesced float4 loads. The next stage's tiles are loaded into registers
// while the current one is multiplied.
template <bool kCodes, int PT, int CT, int BK, bool kCopy = false>
__global__ void __launch_bounds__(NT, kCopy ? 2 : 0) k_project(const float* __restrict__ X, int64_t n_pts, int D,
                                                const float* __restrict__ AT, int lmp, const float* __restrict__ b,
                                                int LM, float W, int32_t* __restrict__ codes,
                                                float* __restrict__ vals, int32_t* __restrict__ pmin,
                                                int32_t* __restrict__ pmax, int* __restrict__ err,
                                                ZeroWords zw, float* __restrict__ xcopy) {
    constexpr int BN = 16 * PT;
    constexpr int BC = 16 * CT;
    constexpr int XP = BN + 2;   // padded X row: the transposing stores conflict at most 4 ways
    constexpr int XS = BN * BK / NT;        // X floats per thread per stage
    constexpr int AV = BC * BK / 4 / NT;    // AT float4 per thread per stage
    static_assert(PT % 2 == 0 && XS % 4 == 0 && AV >= 1 && BC * BK == AV * 4 * NT, "tile shape");
    static_assert(BK % 16 == 0, "As must start 16-byte aligned");
    constexpr int kTileBytes = BK * (XP + BC) * 4;
    constexpr int kStageBytes = BC * (BN + 1) * 4;
    // The epilogue's staging reuses the tiles (the main loop ends on a barrier).
    __shared__ __align__(16) unsigned char smem[kTileBytes > kStageBytes ? kTileBytes : kStageBytes];
    float (*Xs)[XP] = reinterpret_cast<float (*)[XP]>(smem);
    float (*As)[BC] = reinterpret_cast<float (*)[BC]>(smem + BK * XP * 4);
    uint32_t (*Cs)[BN + 1] = reinterpret_cast<uint32_t (*)[BN + 1]>(smem);

    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    zw.clear(tid);
    const int64_t n0 = (int64_t)blockIdx.x * BN;
    const int c0 = blockIdx.y * BC;
    const bool vec = (D & 3) == 0;

    float xr[XS];
    float4 ar[AV];
    // Global -> registers. Vector path: BK/4 consecutive threads read one
    // point's BK dimensions; scalar path (D % 4 != 0): BK threads do. Zero
    // fill past D adds +-0 to a chain, which leaves it unchanged.
    auto gload = [&](int d0) {
        if (vec) {
#pragma unroll
            for (int r = 0; r < XS / 4; ++r) {
                const int f = tid + NT * r, dq = f % (BK / 4), p = f / (BK / 4);
                const int64_t gn = n0 + p;
                const int gd = d0 + dq * 4;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (gn < n_pts && gd < D) {
                    v = __ldg(reinterpret_cast<const float4*>(X + gn * D + gd));
                    if constexpr (kCopy) *reinterpret_cast<float4*>(xcopy + gn * D + gd) = v;
                }
                xr[4 * r + 0] = v.x;
                xr[4 * r + 1] = v.y;
                xr[4 * r + 2] = v.z;
                xr[4 * r + 3] = v.w;
            }
        } else {
#pragma unroll
            for (int r = 0; r < XS; ++r) {
                const int f = tid + NT * r, dd = f % BK, p = f / BK;
                const int64_t gn = n0 + p;
                const int gd = d0 + dd;
                xr[r] = (gn < n_pts && gd < D) ? __ldg(X + gn * D + gd) : 0.0f;
                if constexpr (kCopy) {
                    if (gn < n_pts && gd < D) xcopy[gn * D + gd] = xr[r];
                }
            }
        }
#pragma unroll
        for (int r = 0; r < AV; ++r) {
            const int f = tid + NT * r, cq = f % (BC / 4), dd = f / (BC / 4);
            const int gc = c0 + cq * 4, gd = d0 + dd;
            ar[r] = (gc < lmp && gd < D) ? __ldg(reinterpret_cast<const float4*>(AT + (int64_t)gd * lmp + gc))
                                         : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    auto sstore = [&]() {
        if (vec) {
#pragma unroll
            for (int r = 0; r < XS / 4; ++r) {
                const int f = tid + NT * r, dq = f % (BK / 4), p = f / (BK / 4);
#pragma unroll
                for (int e = 0; e < 4; ++e) Xs[dq * 4 + e][p] = xr[4 * r + e];
            }
        } else {
#pragma unroll
            for (int r = 0; r < XS; ++r) {
                const int f = tid + NT * r, dd = f % BK, p = f / BK;
                Xs[dd][p] = xr[r];
            }
        }
#pragma unroll
        for (int r = 0; r < AV; ++r) {
            const int f = tid + NT * r, cq = f % (BC / 4), dd = f / (BC / 4);
            *reinterpret_cast<float4*>(&As[dd][cq * 4]) = ar[r];
        }
    };

    float acc[PT][CT];
#pragma unroll
    for (int i = 0; i < PT; ++i)
#pragma unroll
        for (int j = 0; j < CT; ++j) acc[i][j] = 0.0f;

    gload(0);
    for (int d0 = 0; d0 < D; d0 += BK) {
        sstore();
        __syncthreads();
        if (d0 + BK < D) gload(d0 + BK);
#pragma unroll 8
        for (int k = 0; k < BK; ++k) {
            float xv[PT];
#pragma unroll
            for (int i = 0; i < PT; i += 2) {
                const float2 x2 = *reinterpret_cast<const float2*>(&Xs[k][16 * i + 2 * tx]);
                xv[i] = x2.x;
                xv[i + 1] = x2.y;
            }
            float aw[CT];
#pragma unroll
            for (int j = 0; j < CT; j += 4) {
                const float4 av = *reinterpret_cast<const float4*>(&As[k][ty * CT + j]);
                aw[j] = av.x;
                aw[j + 1] = av.y;
                aw[j + 2] = av.z;
                aw[j + 3] = av.w;
            }
#pragma unroll
            for (int i = 0; i < PT; ++i)
#pragma unroll
                for (int j = 0; j < CT; ++j) acc[i][j] = __fmaf_rn(xv[i], aw[j], acc[i][j]);
        }
        __syncthreads();
    }

    // Epilogue: -b, /W (IEEE divide), floor; stage through shared memory for
    // coalesced column-major stores.
    int bad = 0;
#pragma unroll
    for (int j = 0; j < CT; ++j) {
        const int c = c0 + ty * CT + j;
        const float bc = (c < LM) ? __ldg(b + c) : 0.0f;
        int32_t lo = INT_MAX, hi = INT_MIN;
#pragma unroll
        for (int i = 0; i < PT; ++i) {
            const int pi = 16 * (i & ~1) + 2 * tx + (i & 1);
            const float v = __fdiv_rn(__fsub_rn(acc[i][j], bc), W);
            uint32_t bits;
            if (kCodes) {
                const float f = floorf(v);
                int32_t code = 0;
                if (!(fabsf(f) <= FLT_MAX)) {
                    bad |= kErrNonFinite;
                } else if (!(f >= -2147483648.0f && f < 2147483648.0f)) {
                    bad |= kErrCodeRange;
                } else {
                    code = (int32_t)f;
                }
                if (n0 + pi < n_pts && c < LM) {
                    lo = min(lo, code);
                    hi = max(hi, code);
                }
                bits = (uint32_t)code;
            } else {
                bits = __float_as_uint(v);
            }
            Cs[ty * CT + j][pi] = bits;
        }
        if (kCodes) {
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) {
                lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
                hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
            }
            if (tx == 0 && c < LM) {
                pmin[(int64_t)blockIdx.x * LM + c] = lo;
                pmax[(int64_t)blockIdx.x * LM + c] = hi;
            }
        }
    }
    if (kCodes && bad) atomicOr(err, bad);
    __syncthreads();
    constexpr int RPI = NT / BN;   // rows stored per iteration
    const int p = tid % BN;
#pragma unroll 4
    for (int r = 0; r < BC / RPI; ++r) {
        const int row = r * RPI + tid / BN;
        const int c = c0 + row;
        if (c < LM && n0 + p < n_pts) {
            const int64_t o = (int64_t)c * n_pts + n0 + p;
            if (kCodes) codes[o] = (int32_t)Cs[row][p];
            else vals[o] = __uint_as_float(Cs[row][p]);
        }
    }
}

__global__ void k_minmax_reduce(const int32_t* __restrict__ pmin, const int32_t* __restrict__ pmax, int nparts, int LM,
                                int32_t* __restrict__ cmin, int32_t* __restrict__ cmax) {
    const int c = blockIdx.x;
    int32_t lo = INT_MAX, hi = INT_MIN;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        lo = min(lo, pmin[(int64_t)i * LM + c]);
        hi = max(hi, pmax[(int64_t)i * LM + c]);
    }
    __shared__ int32_t slo[32], shi[32];
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        slo[w] = lo;
        shi[w] = hi;
    }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        lo = lane < nw ? slo[lane] : INT_MAX;
        hi = lane < nw ? shi[lane] : INT_MIN;
        for (int o = 16; o > 0; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) {
            cmin[c] = lo;
            cmax[c] = hi;
        }
    }
}

}  // namespace

// Index builds (codes) use 128-point tiles; query batches (values) use
// 64-point tiles so that ten thousand queries still fill every SM.
int project_grid_x(int64_t n_pts) { return (int)((n_pts + 127) / 128); }

cudaError_t launch_project_fp32(const float* X, int64_t n_pts, int D, const float* AT, int lmp, const float* b,
                                int LM, float W, int32_t* codes, float* vals, int32_t* pmin, int32_t* pmax, int* err,
                                cudaStream_t st, int tile, ZeroWords zw, float* xcopy) {
    if (n_pts <= 0) return cudaSuccess;
    if (lmp < LM || (lmp & 3) || ((uintptr_t)AT & 15)) return cudaErrorInvalidValue;
    // xcopy (the rows also written to device memory as they are read): one
    // column block, so that every row is read exactly once
    if (xcopy && (codes || tile != 5 || LM > 192)) return cudaErrorInvalidValue;
    if (codes) {
        k_project<true, 8, 4, 16><<<dim3(project_grid_x(n_pts), (LM + 63) / 64), NT, 0, st>>>(
            X, n_pts, D, AT, lmp, b, LM, W, codes, nullptr, pmin, pmax, err, zw, nullptr);
    } else if (tile == 1) {
        k_project<false, 2, 8, 64><<<dim3((unsigned)((n_pts + 31) / 32), (LM + 127) / 128), NT, 0, st>>>(
            X, n_pts, D, AT, lmp, b, LM, W, nullptr, vals, nullptr, nullptr, err, zw, nullptr);
    } else if (tile == 2) {
        k_project<false, 8, 4, 32><<<dim3((unsigned)((n_pts + 127) / 128), (LM + 63) / 64), NT, 0, st>>>(
            X, n_pts, D, AT, lmp, b, LM, W, nullptr, vals, nullptr, nullptr, err, zw, nullptr);
    } else if (tile == 3) {
        k_project<false, 4, 4, 32><<<dim3((unsigned)((n_pts + 63) / 64), (LM + 63) / 64), NT, 0, st>>>(
            X, n_pts, D, AT, lmp, b, LM, W, nullptr, vals, nullptr, nullptr, err, zw, nullptr);
    } else if (tile == 4) {
        k_project<false, 2, 4, 32><<<dim3((unsigned)((n_pts + 31) / 32), (LM + 63) / 64), NT, 0, st>>>(
            X, n_pts, D, AT, lmp, b, LM, W, nullptr, vals, nullptr, nullptr, err, zw, nullptr);
    } else if (tile == 5) {
        if (!xcopy) return cudaErrorInvalidValue;   // tiling 5 serves the copying form only
        k_project<false, 2, 12, 32, true><<<dim3((unsigned)((n_pts + 31) / 32), (LM + 191) / 192), NT, 0, st>>>(
            X, n_pts, D, AT, lmp, b, LM, W, nullptr, vals, nullptr, nullptr, err, zw, xcopy);
    } else {
        k_project<false, 4, 8, 32><<<dim3((unsigned)((n_pts + 63) / 64), (LM + 127) / 128), NT, 0, st>>>(
            X, n_pts, D, AT, lmp, b, LM, W, nullptr, vals, nullptr, nullptr, err, zw, nullptr);
    }
    return cudaGetLastError();
}

template <typename F>
struct arity;
template <typename R, typename... A>
struct arity<R(A...)> {
    static constexpr int value = sizeof...(A);
};
static_assert(arity<decltype(k_project<false, 2, 12, 32, true>)>::value == kProjectArgs, "projection parameters");

const void* project_copy_kernel() { return reinterpret_cast<const void*>(&k_project<false, 2, 12, 32, true>); }

cudaError_t launch_minmax_reduce(const int32_t* pmin, const int32_t* pmax, int nparts, int LM, int32_t* cmin,
                                 int32_t* cmax, cudaStream_t st) {
    k_minmax_reduce<<<LM, 256, 0, st>>>(pmin, pmax, nparts, LM, cmin, cmax);
    return cudaGetLastError();
}

// Copies n floats from src (16-byte aligned; host memory the device can read,
// or device memory) to dst with 16-byte loads: one pass over the source. Each
// thread issues kCopyVec independent loads before its stores, so that reads
// over the host link (microseconds of latency) overlap.
constexpr int kCopyVec = 8;

__global__ void __launch_bounds__(256) k_copy_f32(const float* __restrict__ src, float* __restrict__ dst, int64_t n) {
    const int64_t n4 = n >> 2;
    const float4* s4 = reinterpret_cast<const float4*>(src);
    float4* d4 = reinterpret_cast<float4*>(dst);
    const int64_t base = (int64_t)blockIdx.x * (256 * kCopyVec) + threadIdx.x;
    float4 v[kCopyVec];
#pragma unroll
    for (int k = 0; k < kCopyVec; ++k) {
        const int64_t i = base + (int64_t)k * 256;
        if (i < n4) v[k] = s4[i];
    }
#pragma unroll
    for (int k = 0; k < kCopyVec; ++k) {
        const int64_t i = base + (int64_t)k * 256;
        if (i < n4) d4[i] = v[k];
    }
    if (blockIdx.x == 0 && threadIdx.x < (n & 3)) dst[(n4 << 2) + threadIdx.x] = src[(n4 << 2) + threadIdx.x];
}

cudaError_t launch_copy_f32(const float* src, float* dst, int64_t n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (((uintptr_t)src & 15) || ((uintptr_t)dst & 15)) return cudaErrorInvalidValue;
    const int64_t blocks = ((n >> 2) + 256 * kCopyVec - 1) / (256 * kCopyVec);
    k_copy_f32<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

}  // namespace culsh
