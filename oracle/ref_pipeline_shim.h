/* Host build of the reference's whole index and search path, for pinning the
 * oracle end to end (tests/test_oracle_refpipeline.py). The reference's five
 * source files (cuLSH_Kernels.cu, cuLSH_Indexing.cu, cuLSH_Querying.cu,
 * cuLSH_HashTables.cu, cuLSH_SearchTables.cu, in the order cuLSH.h:93-97
 * includes them) are read from where they lie and fed to the host compiler
 * through a pipe; the one edit on the way is the kernel launch syntax,
 * `kernel <<< grid, block >>> (args)` becoming `REF_LAUNCH(kernel, grid,
 * block)(args)` (see the Makefile's `ref` target). This header is
 * force-included before them and stands in for cuLSH.h:22-90:
 *
 * - Thrust's CPP backend, so that thrust::device_vector lives in host memory
 *   and every Thrust algorithm of the reference runs on the host;
 * - the CUDA kernel keywords, thread indices and intrinsics of ref_shim.h
 *   (the same header the kernel-only build uses), a dim3, and launchers
 *   that run a grid as loops on the host: a kernel that shares nothing
 *   between threads runs one thread after another; kernel_calculateDistances
 *   (__shared__ + __syncthreads) runs each block on one host thread per CUDA
 *   thread meeting at a barrier;
 * - stand-ins for the closed libraries: cublasSgemm is the oracle's own
 *   canonical FMA chain for X'A (ref_pipeline_host.cpp), cuRAND is absent
 *   (the random reset fails; the tests set A and b), CUDA events time
 *   nothing, and cuMemGetInfo reports a free-memory figure the caller sets,
 *   which drives the reference's query chunking (cuLSH_SearchTables.cu:282-306);
 * - the reference's device_vector typedefs over an allocator that keeps 64
 *   spare elements past every allocation: kernel_calculateDistances writes a
 *   result for every row of its last block, in range or not
 *   (cuLSH_Kernels.cu:346), which on a GPU lands in slack memory and on the
 *   host would corrupt the heap. */
#ifndef CULSH_REF_PIPELINE_SHIM_H
#define CULSH_REF_PIPELINE_SHIM_H

#define THRUST_DEVICE_SYSTEM THRUST_DEVICE_SYSTEM_CPP

#include <barrier>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <iterator>
#include <thread>
#include <vector>

#include <thrust/adjacent_difference.h>
#include <thrust/copy.h>
#include <thrust/count.h>
#include <thrust/device_allocator.h>
#include <thrust/device_vector.h>
#include <thrust/extrema.h>
#include <thrust/fill.h>
#include <thrust/gather.h>
#include <thrust/host_vector.h>
#include <thrust/iterator/constant_iterator.h>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/permutation_iterator.h>
#include <thrust/iterator/transform_iterator.h>
#include <thrust/reduce.h>
#include <thrust/scan.h>
#include <thrust/scatter.h>
#include <thrust/sequence.h>
#include <thrust/sort.h>
#include <thrust/transform.h>
#include <thrust/unique.h>

#include "ref_shim.h"
#ifndef __host__
#define __host__
#endif

#define BLOCK_SIZE 16
#define DEF_MB(x) ((x) / (float)(1 << 20))
#define DEF_SECONDS(x) ((x) / (float)CLOCKS_PER_SEC)
#define DEF_PRINT_ERROR(...) do { fprintf(stderr, "[reference error] "); fprintf(stderr, __VA_ARGS__); } while (0)

template <class T>
struct ref_padded_allocator : thrust::device_allocator<T> {
    using base = thrust::device_allocator<T>;
    static constexpr size_t kSpare = 64;
    template <class U>
    struct rebind {
        using other = ref_padded_allocator<U>;
    };
    ref_padded_allocator() = default;
    template <class U>
    ref_padded_allocator(const ref_padded_allocator<U>&) {}
    typename base::pointer allocate(size_t n) { return base::allocate(n + kSpare); }
    void deallocate(typename base::pointer p, size_t n) { base::deallocate(p, n + kSpare); }
};

typedef thrust::device_vector<float, ref_padded_allocator<float>> ThrustFloatD;
typedef thrust::device_vector<unsigned, ref_padded_allocator<unsigned>> ThrustUnsignedD;
typedef thrust::device_vector<int, ref_padded_allocator<int>> ThrustIntD;
typedef thrust::device_vector<uint64_t, ref_padded_allocator<uint64_t>> ThrustUint64D;
typedef thrust::host_vector<float> ThrustFloatH;
typedef thrust::host_vector<unsigned> ThrustUnsignedH;
typedef thrust::host_vector<int> ThrustIntH;
typedef thrust::host_vector<uint64_t> ThrustUint64H;

struct dim3 {
    unsigned x, y, z;
    dim3(unsigned x_ = 1, unsigned y_ = 1, unsigned z_ = 1) : x(x_), y(y_), z(z_) {}
};

/* ---- launches ---- */
extern thread_local std::barrier<>* ref_block_barrier;
void ref_block_sync();

template <class F>
void ref_run_serial(dim3 grid, dim3 block, F body) {
    gridDim = ref_dim3{grid.x, grid.y, grid.z};
    blockDim = ref_dim3{block.x, block.y, block.z};
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

/* One host thread per CUDA thread of a block, all blocks in turn; a barrier
 * after each block keeps the next block's writes to the kernel's static
 * "shared" array behind the previous block's last reads. */
template <class F>
void ref_run_blocks(dim3 grid, dim3 block, F body) {
    const unsigned nt = block.x * block.y * block.z;
    std::barrier<> bar((std::ptrdiff_t)nt);
    std::vector<std::thread> threads;
    threads.reserve(nt);
    for (unsigned t = 0; t < nt; ++t)
        threads.emplace_back([&, t] {
            gridDim = ref_dim3{grid.x, grid.y, grid.z};
            blockDim = ref_dim3{block.x, block.y, block.z};
            threadIdx = ref_dim3{t % block.x, (t / block.x) % block.y, t / (block.x * block.y)};
            ref_block_barrier = &bar;
            ref_sync_hook = ref_block_sync;
            for (unsigned bz = 0; bz < grid.z; ++bz)
                for (unsigned by = 0; by < grid.y; ++by)
                    for (unsigned bx = 0; bx < grid.x; ++bx) {
                        blockIdx = ref_dim3{bx, by, bz};
                        body();
                        bar.arrive_and_wait();
                    }
            ref_sync_hook = nullptr;
            ref_block_barrier = nullptr;
        });
    for (auto& th : threads) th.join();
}

template <class K>
struct ref_launcher {
    K kernel;
    dim3 grid, block;
    const char* name;
    template <class... A>
    void operator()(A... args) const {
        auto body = [&] { kernel(args...); };
        if (std::strcmp(name, "kernel_calculateDistances") == 0)
            ref_run_blocks(grid, block, body);
        else
            ref_run_serial(grid, block, body);
    }
};
#define REF_LAUNCH(k, g, b) ref_launcher<decltype(&k)>{&k, (g), (b), #k}

/* ---- CUDA runtime and driver calls the reference makes ---- */
typedef int cudaEvent_t;
static inline int cudaEventCreate(cudaEvent_t* e) { *e = 0; return 0; }
static inline int cudaEventRecord(cudaEvent_t) { return 0; }
static inline int cudaEventSynchronize(cudaEvent_t) { return 0; }
static inline int cudaEventElapsedTime(float* ms, cudaEvent_t, cudaEvent_t) { *ms = 0.0f; return 0; }
static inline int cudaEventDestroy(cudaEvent_t) { return 0; }
static inline int cudaDeviceSynchronize() { return 0; }
static inline int cudaProfilerStart() { return 0; }
static inline int cudaProfilerStop() { return 0; }
extern size_t ref_free_bytes;
static inline int cuMemGetInfo(size_t* free_b, size_t* total_b) {
    *free_b = ref_free_bytes;
    *total_b = ref_free_bytes;
    return 0;
}

/* ---- cuBLAS: the one GEMM (defined in ref_pipeline_host.cpp) ---- */
typedef void* cublasHandle_t;
enum cublasStatus_t { CUBLAS_STATUS_SUCCESS = 0, CUBLAS_STATUS_NOT_SUPPORTED = 15 };
enum cublasOperation_t { CUBLAS_OP_N = 0, CUBLAS_OP_T = 1 };
static inline cublasStatus_t cublasCreate(cublasHandle_t* h) { *h = nullptr; return CUBLAS_STATUS_SUCCESS; }
cublasStatus_t cublasSgemm(cublasHandle_t, cublasOperation_t, cublasOperation_t, int m, int n, int k,
                           const float* alpha, const float* A, int lda, const float* B, int ldb, const float* beta,
                           float* C, int ldc);

/* ---- cuRAND: not available (reset with explicit A and b only) ---- */
typedef void* curandGenerator_t;
enum curandStatus_t { CURAND_STATUS_SUCCESS = 0, CURAND_STATUS_NOT_INITIALIZED = 201 };
enum curandRngType_t { CURAND_RNG_PSEUDO_DEFAULT = 100 };
static inline curandStatus_t curandCreateGenerator(curandGenerator_t*, curandRngType_t) {
    return CURAND_STATUS_NOT_INITIALIZED;
}
static inline curandStatus_t curandSetPseudoRandomGeneratorSeed(curandGenerator_t, unsigned long long) {
    return CURAND_STATUS_NOT_INITIALIZED;
}
static inline curandStatus_t curandGenerateUniform(curandGenerator_t, float*, size_t) {
    return CURAND_STATUS_NOT_INITIALIZED;
}
static inline curandStatus_t curandGenerateNormal(curandGenerator_t, float*, size_t, float, float) {
    return CURAND_STATUS_NOT_INITIALIZED;
}
static inline curandStatus_t curandDestroyGenerator(curandGenerator_t) { return CURAND_STATUS_NOT_INITIALIZED; }

#endif
