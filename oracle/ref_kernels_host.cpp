// Runs the reference's own kernels (cuLSH_Kernels.cu, compiled for the host
// through ref_shim.h from the reference tree, see the Makefile's `ref`
// target) on host arrays, with the buffer preparation and launch shapes of
// the reference's host code, so that the tests can check the oracle against
// the reference itself. Test infrastructure only: nothing in the library
// links or loads it.
//
// Entry points (extern "C"):
//   ref_projection_epilogue  kernel_subtractVectorFromMatrixRows,
//                            kernel_divideMatrixWithScalar, kernel_floorMatrix
//                            as cuLSH_Indexing.cu:53-66 launches them
//   ref_probing_codes        kernel_calculateDeltas + kernel_calculateProbingCodes
//                            with the row layout of createMultiprobingCodes
//                            (cuLSH_Querying.cu:63-119)
//   ref_topk                 kernel_configureIds + kernel_sortIds as
//                            calculateIds launches them (cuLSH_Querying.cu:231-277)
//   ref_distances            kernel_calculateDistances as calculateDistances
//                            launches it (cuLSH_Querying.cu:284-343)
//
// The file is compiled with floating-point contraction on, as nvcc's default
// (-fmad=true) compiles the reference: its one multiply feeding an add, the
// distance accumulation, becomes a fused multiply-add on both.
#include "cuLSH_Kernels.cu"

#include <barrier>
#include <thread>
#include <vector>

thread_local ref_dim3 threadIdx, blockIdx, blockDim, gridDim;
thread_local void (*ref_sync_hook)() = nullptr;

namespace {

constexpr unsigned kBlock = 16;   // BLOCK_SIZE of cuLSH.h:71

// One launch: the body runs once per thread of the grid, in order.
template <class F>
void launch(ref_dim3 grid, ref_dim3 block, F body) {
    gridDim = grid;
    blockDim = block;
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                blockIdx = ref_dim3{bx, by, bz};
                for (unsigned tz = 0; tz < block.z; ++tz)
                    for (unsigned ty = 0; ty < block.y; ++ty)
                        for (unsigned tx = 0; tx < block.x; ++tx) {
                            threadIdx = ref_dim3{tx, ty, tz};
                            body();
                        }
            }
}

unsigned cdiv(unsigned a, unsigned b) { return (a + b - 1) / b; }

// A launch whose blocks synchronise: each block runs as one host thread per
// CUDA thread, blocks one after another, __syncthreads() on the block's
// barrier (every thread of the reference kernel reaches each one).
std::barrier<>* g_block_barrier = nullptr;
void block_sync() { g_block_barrier->arrive_and_wait(); }

template <class F>
void launch_cooperative(ref_dim3 grid, ref_dim3 block, F body) {
    const unsigned nt = block.x * block.y * block.z;
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx) {
                std::barrier<> bar((std::ptrdiff_t)nt);
                g_block_barrier = &bar;
                std::vector<std::thread> threads;
                threads.reserve(nt);
                for (unsigned tz = 0; tz < block.z; ++tz)
                    for (unsigned ty = 0; ty < block.y; ++ty)
                        for (unsigned tx = 0; tx < block.x; ++tx)
                            threads.emplace_back([&, tx, ty, tz, bx, by, bz] {
                                gridDim = grid;
                                blockDim = block;
                                blockIdx = ref_dim3{bx, by, bz};
                                threadIdx = ref_dim3{tx, ty, tz};
                                ref_sync_hook = block_sync;
                                body();
                                ref_sync_hook = nullptr;
                            });
                for (auto& t : threads) t.join();
                g_block_barrier = nullptr;
            }
}

}  // namespace

extern "C" {

// C: rows x cols column-major (element (r, c) at c*rows + r), the projections
// X'A; replaced by fl(fl(C - b[c]) / W), floored when do_floor.
int ref_projection_epilogue(float* C, int rows, int cols, const float* b, float W, int do_floor) {
    if (rows <= 0 || cols <= 0) return -1;
    const ref_dim3 block{kBlock, kBlock, 1}, grid{cdiv(rows, kBlock), cdiv(cols, kBlock), 1};
    launch(grid, block, [&] { cuLSH::kernel_subtractVectorFromMatrixRows(C, b, rows, cols); });
    launch(grid, block, [&] { cuLSH::kernel_divideMatrixWithScalar(C, W, rows, cols); });
    if (do_floor) launch(grid, block, [&] { cuLSH::kernel_floorMatrix(C, rows, cols); });
    return 0;
}

// vals: the non-floored projections of Q queries on one table, column-major
// (value of column m for query q at m*Q + q). out: the Q*T probe codes of the
// table, column-major over (Q*T) rows, row q*T + t (value at m*Q*T + q*T + t),
// as the reference leaves them for the bucket match. M <= 15: the kernel tests
// mask bits with a 32-bit `1 << i`, defined only below bit 31.
int ref_probing_codes(const float* vals, int Q, int M, int T, float* out) {
    if (Q <= 0 || M <= 0 || M > 15 || T <= 0) return -1;
    std::vector<float> proj(vals, vals + (size_t)Q * M), deltas((size_t)Q * 2 * M);
    launch(ref_dim3{cdiv(Q, kBlock), cdiv(M, kBlock), 1}, ref_dim3{kBlock, kBlock, 1},
           [&] { cuLSH::kernel_calculateDeltas(proj.data(), Q, M, deltas.data()); });
    // row q*T of each column holds the (now floored) home code, the rest 0
    std::vector<float> mp((size_t)Q * T * M, 0.0f);
    for (int m = 0; m < M; ++m)
        for (int q = 0; q < Q; ++q) mp[(size_t)m * Q * T + (size_t)q * T] = proj[(size_t)m * Q + q];
    std::vector<uint64_t> comb((size_t)Q * T, 0);
    std::vector<float> comb_d((size_t)Q * T, 0.0f);
    launch(ref_dim3{cdiv(Q, kBlock * kBlock), 1, 1}, ref_dim3{kBlock * kBlock, 1, 1}, [&] {
        cuLSH::kernel_calculateProbingCodes(mp.data(), Q, M, T, deltas.data(), comb.data(), comb_d.data());
    });
    for (size_t i = 0; i < mp.size(); ++i) out[i] = mp[i];
    return 0;
}

// Candidates of Q queries: query q owns ids[starts[q] .. starts[q]+sizes[q])
// with distances dist[...] at the same positions (total entries in all).
// out_ids / out_d: Q*K, query q's K nearest at q*K .. q*K+K-1, padded with
// (-1, FLT_MAX).
int ref_topk(int Q, int K, const unsigned* ids, const unsigned* starts, const unsigned* sizes, unsigned total,
             const float* dist, int* out_ids, float* out_d) {
    if (Q <= 0 || K <= 0) return -1;
    for (size_t i = 0; i < (size_t)Q * K; ++i) {
        out_d[i] = FLT_MAX;
        out_ids[i] = -1;
    }
    const ref_dim3 block{kBlock * kBlock, 1, 1}, grid{cdiv(Q, kBlock * kBlock), 1, 1};
    launch(grid, block, [&] { cuLSH::kernel_configureIds(out_d, out_ids, Q, K, total, dist, ids, starts, sizes); });
    launch(grid, block, [&] { cuLSH::kernel_sortIds(out_d, out_ids, Q, K); });
    return 0;
}

// Squared L2 distance of each (query qidx[i], point cand[i]) pair, i < total;
// queries Q x D and data N x D row-major (point-contiguous). One launch of up
// to 65535 * 32 pairs, as the reference chunks them.
int ref_distances(const float* queries, int D, int Q, const float* data, int N, const unsigned* cand,
                  const unsigned* qidx, unsigned total, float* out) {
    if (D <= 0 || total > 65535u * BLOCK_SIZE_Y) return -1;
    if (total == 0) return 0;
    const unsigned nb = cdiv(total, BLOCK_SIZE_Y);
    // the kernel writes a result for every row of its last block, in range or not
    std::vector<float> d((size_t)nb * BLOCK_SIZE_Y, 0.0f);
    launch_cooperative(ref_dim3{1, nb, 1}, ref_dim3{BLOCK_SIZE_REDUCE, BLOCK_SIZE_Y, 1}, [&] {
        cuLSH::kernel_calculateDistances(d.data(), total, queries, D, Q, data, N, cand, qidx);
    });
    for (unsigned i = 0; i < total; ++i) out[i] = d[i];
    return 0;
}

}  // extern "C"
