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
#include <cfloat>
#include <climits>

#include "culsh_internal.cuh"

namespace culsh {
namespace {

constexpr int BN = 128;   // points per block tile
constexpr int BC = 64;    // projection columns per block tile
constexpr int BK = 16;    // dimensions per shared-memory stage
constexpr int NT = 256;   // threads: 16 (points) x 16 (columns), each 8 x 4 outputs

template <bool kCodes>
__global__ void __launch_bounds__(NT) k_project(const float* __restrict__ X, int64_t n_pts, int D,
                                                const float* __restrict__ A, const float* __restrict__ b, int LM,
                                                float W, int32_t* __restrict__ codes, float* __restrict__ vals,
                                                int32_t* __restrict__ pmin, int32_t* __restrict__ pmax,
                                                int* __restrict__ err) {
    __shared__ __align__(16) float Xs[BK][BN];
    __shared__ __align__(16) float As[BK][BC];
    __shared__ uint32_t Cs[BC][BN + 1];

    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int64_t n0 = (int64_t)blockIdx.x * BN;
    const int c0 = blockIdx.y * BC;
    const bool vec = (D & 3) == 0;

    float acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;

    for (int d0 = 0; d0 < D; d0 += BK) {
        // X tile: 128 points x 16 dims, transposed into Xs[dim][point]. Zero
        // fill past D adds +-0 to a chain, which leaves it unchanged.
        if (vec) {
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const int f = tid + NT * r, p = f & (BN - 1), dq = f >> 7;
                const int64_t gn = n0 + p;
                const int gd = d0 + dq * 4;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (gn < n_pts && gd < D) v = __ldg(reinterpret_cast<const float4*>(X + gn * D + gd));
                Xs[dq * 4 + 0][p] = v.x;
                Xs[dq * 4 + 1][p] = v.y;
                Xs[dq * 4 + 2][p] = v.z;
                Xs[dq * 4 + 3][p] = v.w;
            }
        } else {
#pragma unroll
            for (int r = 0; r < 8; ++r) {
                const int f = tid + NT * r, p = f & (BN - 1), dd = f >> 7;
                const int64_t gn = n0 + p;
                const int gd = d0 + dd;
                Xs[dd][p] = (gn < n_pts && gd < D) ? __ldg(X + gn * D + gd) : 0.0f;
            }
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int f = tid + NT * r, c = f & (BC - 1), dd = f >> 6;
            const int gc = c0 + c, gd = d0 + dd;
            As[dd][c] = (gc < LM && gd < D) ? __ldg(A + (int64_t)gc * D + gd) : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            const float4 xa = *reinterpret_cast<const float4*>(&Xs[k][tx * 8]);
            const float4 xb = *reinterpret_cast<const float4*>(&Xs[k][tx * 8 + 4]);
            const float4 av = *reinterpret_cast<const float4*>(&As[k][ty * 4]);
            const float xv[8] = {xa.x, xa.y, xa.z, xa.w, xb.x, xb.y, xb.z, xb.w};
            const float aw[4] = {av.x, av.y, av.z, av.w};
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = __fmaf_rn(xv[i], aw[j], acc[i][j]);
        }
        __syncthreads();
    }

    // Epilogue: -b, /W (IEEE divide), floor; stage through shared memory for
    // coalesced column-major stores.
    int bad = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int c = c0 + ty * 4 + j;
        const float bc = (c < LM) ? __ldg(b + c) : 0.0f;
        int32_t lo = INT_MAX, hi = INT_MIN;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
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
                if (n0 + tx * 8 + i < n_pts && c < LM) {
                    lo = min(lo, code);
                    hi = max(hi, code);
                }
                bits = (uint32_t)code;
            } else {
                bits = __float_as_uint(v);
            }
            Cs[ty * 4 + j][tx * 8 + i] = bits;
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
    const int p = tid & (BN - 1);
#pragma unroll 4
    for (int r = 0; r < BC / 2; ++r) {
        const int row = r * 2 + (tid >> 7);
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

int project_grid_x(int64_t n_pts) { return (int)((n_pts + BN - 1) / BN); }

cudaError_t launch_project_fp32(const float* X, int64_t n_pts, int D, const float* A, const float* b, int LM,
                                float W, int32_t* codes, float* vals, int32_t* pmin, int32_t* pmax, int* err,
                                cudaStream_t st) {
    if (n_pts <= 0) return cudaSuccess;
    const dim3 grid(project_grid_x(n_pts), (LM + BC - 1) / BC);
    if (codes)
        k_project<true><<<grid, NT, 0, st>>>(X, n_pts, D, A, b, LM, W, codes, nullptr, pmin, pmax, err);
    else
        k_project<false><<<grid, NT, 0, st>>>(X, n_pts, D, A, b, LM, W, nullptr, vals, nullptr, nullptr, err);
    return cudaGetLastError();
}

cudaError_t launch_minmax_reduce(const int32_t* pmin, const int32_t* pmax, int nparts, int LM, int32_t* cmin,
                                 int32_t* cmax, cudaStream_t st) {
    k_minmax_reduce<<<LM, 256, 0, st>>>(pmin, pmax, nparts, LM, cmin, cmax);
    return cudaGetLastError();
}

}  // namespace culsh
