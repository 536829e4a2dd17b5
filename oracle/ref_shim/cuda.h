/*
 * Stand-in for <cuda.h> / <cuda_runtime.h> used ONLY to compile the
 * reference's own src/kernels.cu and src/wavefront.cuh as host C++ for the
 * CPU oracle in oracle/_ref (test infrastructure, never shipped).
 *
 * It models one CUDA thread block executed by a single host thread: the
 * kernels are called with blockDim = (1,1,1), so every block-strided loop of
 * the reference runs all of its iterations in one thread.  For the reference
 * kernels that is exact: each wavefront step reads one buffer and writes the
 * other (src/kernels.cu:111-180), so the order of the diagonals inside a
 * step does not matter, and __syncthreads() has nothing left to order.
 * Runtime calls are never reached by the oracle; they fail with an error
 * code instead of touching a GPU.
 */
#ifndef WFE_REF_SHIM_CUDA_H
#define WFE_REF_SHIM_CUDA_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <algorithm>

typedef int cudaError_t;
typedef void* cudaStream_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2 };

static inline cudaError_t cudaMalloc(void** p, size_t) { *p = NULL; return 2; }
static inline cudaError_t cudaMallocHost(void** p, size_t) { *p = NULL; return 2; }
static inline cudaError_t cudaFree(void*) { return 2; }
static inline cudaError_t cudaMemset(void*, int, size_t) { return 2; }
static inline cudaError_t cudaMemsetAsync(void*, int, size_t, cudaStream_t) { return 2; }
static inline cudaError_t cudaMemcpy(void*, const void*, size_t, cudaMemcpyKind) { return 2; }
static inline cudaError_t cudaMemcpyAsync(void*, const void*, size_t, cudaMemcpyKind, cudaStream_t) { return 2; }
static inline cudaError_t cudaStreamCreate(cudaStream_t*) { return 2; }
/* The reference checks errors with cudaGetLastError(); report success so that
 * constructing its Cigars helper object does not exit the process. */
static inline cudaError_t cudaGetLastError() { return cudaSuccess; }
static inline const char* cudaGetErrorName(cudaError_t) { return "shim"; }
static inline const char* cudaGetErrorString(cudaError_t) { return "shim"; }

struct wfe_shim_dim3 { unsigned x, y, z; };
extern wfe_shim_dim3 threadIdx, blockIdx, blockDim;

#define __global__
#define __device__
#define __host__
#define __shared__
static inline void __syncthreads() {}
static inline int __clz(unsigned x) { return x ? __builtin_clz(x) : 32; }
using std::max;
using std::min;

#endif
