/* Host build of the reference's own kernel file (cuLSH_Kernels.cu, included
 * from where it lies, never copied) for pinning the oracle: this header is
 * force-included before it and makes its CUDA C compile as plain C++.
 *
 * Test infrastructure only (tests/test_oracle_refkernels.py). A kernel runs
 * as a loop over its grid that calls the kernel body once per thread with
 * blockIdx/threadIdx set (ref_kernels_host.cpp), which is exact for kernels
 * that share nothing between threads. kernel_calculateDistances (shared memory
 * + __syncthreads) runs each block as one host thread per CUDA thread: its
 * __shared__ array becomes a function-local static, and __syncthreads() waits
 * on the block's barrier through ref_sync_hook.
 *
 * The three macros below are the values cuLSH.h:71-77 gives them; that header
 * itself needs the CUDA libraries and is not included. */
#ifndef CULSH_REF_SHIM_H
#define CULSH_REF_SHIM_H

#include <cfloat>
#include <cmath>
#include <cstdint>

#define __global__
#define __device__
#define __shared__ static

#define BLOCK_SIZE_REDUCE 8
#define BLOCK_SIZE_Y 32
#define DEF_MIN(x, y) (((x) < (y)) ? (x) : (y))

struct ref_dim3 {
    unsigned x, y, z;
};
extern thread_local ref_dim3 threadIdx, blockIdx, blockDim, gridDim;

extern thread_local void (*ref_sync_hook)();
static inline void __syncthreads() {
    if (ref_sync_hook) ref_sync_hook();
}
/* Round toward +infinity to int / unsigned. The arguments here are
 * log2f(n) of small positive n, where that is the ceiling. */
static inline int __float2int_ru(float x) { return (int)std::ceil(x); }
static inline unsigned __float2uint_ru(float x) { return (unsigned)std::ceil(x); }
static inline int __clzll(long long x) { return x ? __builtin_clzll((unsigned long long)x) : 64; }

#endif
