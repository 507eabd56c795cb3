/*
 * md_device.cuh -- device helpers shared by the kernel files.
 */
#ifndef MD_DEVICE_CUH
#define MD_DEVICE_CUH

#include "md_internal.h"

/* FP32 minimum-image r^2 with every operation rounded separately, exactly as
 * neighborlist.cu:268-283 (and :167-174) write it: no FMA contraction, so the
 * neighbour set and the rebuild decision are bit-identical to the reference's
 * on the same positions. */
__device__ __forceinline__ float md_rsq_exact(float4 a, float4 b, const md_kparams &kp)
{
    float dx = __fsub_rn(a.x, b.x);
    float dy = __fsub_rn(a.y, b.y);
    float dz = __fsub_rn(a.z, b.z);
    dx = __fsub_rn(dx, __fmul_rn(kp.box[0], rintf(__fmul_rn(dx, kp.boxi[0]))));
    dy = __fsub_rn(dy, __fmul_rn(kp.box[1], rintf(__fmul_rn(dy, kp.boxi[1]))));
    dz = __fsub_rn(dz, __fmul_rn(kp.box[2], rintf(__fmul_rn(dz, kp.boxi[2]))));
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

/* True in every thread of the block that finishes last (threadfence
 * reduction).  The caller's prior global writes are visible to that block;
 * it must read other blocks' results with __ldcg / volatile and reset the
 * counter. */
__device__ __forceinline__ bool md_last_block(unsigned *counter)
{
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
    __syncthreads();
    return last;
}

#endif
