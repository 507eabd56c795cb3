/*
 * cuda_shim.h -- lets g++ compile the reference's CUDA kernel files as host
 * C++ so that they run on the CPU (the role the reference's own -deviceemu
 * build target once played, src/Makefile:42).  TEST INFRASTRUCTURE: used only
 * to produce golden vectors that pin the oracle.
 *
 * Execution-space qualifiers vanish, the builtin index variables become
 * globals set by a fiber scheduler (ref_fibers.cpp), and __syncthreads()
 * yields to that scheduler so every thread of a block reaches the barrier
 * before any continues.  Device intrinsics get IEEE host definitions:
 * rsqrtf(x) = 1/sqrtf(x), __fdividef(a,b) = a/b; exp2f/acosf/rintf/truncf
 * are the C library's.  The same definitions are used by the oracle's
 * "as written" FP32 mode, so the two must agree bit for bit.
 */
#ifndef REF_CUDA_SHIM_H
#define REF_CUDA_SHIM_H

#include <cuda_runtime.h>
#include <vector_functions.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define __global__
#define __device__
#define __constant__
#define __shared__

extern uint3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;

void __syncthreads(void);

static inline int __mul24(int a, int b) { return a * b; }
static inline float rsqrtf(float x) { return 1.0f / sqrtf(x); }
static inline float __fdividef(float a, float b) { return a / b; }
static inline int __float2int_rd(float x) { return (int)floorf(x); }
static inline float __int2float_rd(int i) { return (float)i; }
static inline int min(int a, int b) { return a < b ? a : b; }

/* Legacy texture reference: a read-only view of a float4 array. */
template <class T, int D, int M>
struct texture {
    const T *ptr;
};
template <class T, int D, int M>
static inline T tex1Dfetch(const texture<T, D, M> &t, int i) { return t.ptr[i]; }

#endif
