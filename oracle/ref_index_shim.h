/* Host build of the reference's own index-side host code for pinning the
 * oracle (tests/test_oracle_refkernels.py): the row sort and bucket
 * boundaries of cuLSH_Indexing.cu:71-144 and the index file reader and writer
 * of cuLSH_HashTables.cu:51-119,251-483, read from where they lie and fed to
 * the compiler through a pipe (never copied; see the Makefile's `ref`
 * target). This header is force-included before them: it selects Thrust's
 * CPP backend, so that their thrust::device_vector objects live in host memory
 * and their Thrust algorithms run on the host, and gives the names they take
 * from cuLSH.h (cuLSH.h:79-83) equivalents that need no CUDA library. */
#ifndef CULSH_REF_INDEX_SHIM_H
#define CULSH_REF_INDEX_SHIM_H

#define THRUST_DEVICE_SYSTEM THRUST_DEVICE_SYSTEM_CPP

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include <thrust/adjacent_difference.h>
#include <thrust/copy.h>
#include <thrust/count.h>
#include <thrust/device_vector.h>
#include <thrust/fill.h>
#include <thrust/gather.h>
#include <thrust/host_vector.h>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/sequence.h>
#include <thrust/sort.h>
#include <thrust/transform.h>

#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif

typedef thrust::device_vector<float> ThrustFloatD;
typedef thrust::device_vector<unsigned> ThrustUnsignedD;
#define DEF_PRINT_ERROR(...) do { printf("[reference error] "); printf(__VA_ARGS__); } while (0)

#endif
