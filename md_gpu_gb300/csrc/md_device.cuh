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
__device__ __forceinline__ float md_rsq_box(float4 a, float4 b, const float *box,
                                            const float *boxi)
{
    float dx = __fsub_rn(a.x, b.x);
    float dy = __fsub_rn(a.y, b.y);
    float dz = __fsub_rn(a.z, b.z);
    dx = __fsub_rn(dx, __fmul_rn(box[0], rintf(__fmul_rn(dx, boxi[0]))));
    dy = __fsub_rn(dy, __fmul_rn(box[1], rintf(__fmul_rn(dy, boxi[1]))));
    dz = __fsub_rn(dz, __fmul_rn(box[2], rintf(__fmul_rn(dz, boxi[2]))));
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

__device__ __forceinline__ float md_rsq_exact(float4 a, float4 b, const md_kparams &kp)
{
    return md_rsq_box(a, b, kp.box, kp.boxi);
}

/* Two FP32 lanes in one 64-bit register pair: the sm_100+ packed
 * instructions add/sub/mul/fma.rn.f32x2 compute two entries' operations in
 * one issue slot, each half rounded as the scalar instruction would. */
typedef unsigned long long f32x2;
template <bool PACKED>
struct v2;
template <>
struct v2<true> {
    f32x2 d;
    __device__ __forceinline__ static v2 make(float a, float b)
    {
        v2 r;
        asm("mov.b64 %0, {%1, %2};" : "=l"(r.d) : "f"(a), "f"(b));
        return r;
    }
    __device__ __forceinline__ void get(float &a, float &b) const
    {
        asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(d));
    }
    __device__ __forceinline__ friend v2 operator+(v2 a, v2 b)
    {
        v2 r;
        asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.d) : "l"(a.d), "l"(b.d));
        return r;
    }
    __device__ __forceinline__ friend v2 operator-(v2 a, v2 b)
    {
        v2 r;
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.d) : "l"(a.d), "l"(b.d));
        return r;
    }
    __device__ __forceinline__ friend v2 operator*(v2 a, v2 b)
    {
        v2 r;
        asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.d) : "l"(a.d), "l"(b.d));
        return r;
    }
    __device__ __forceinline__ static v2 fma(v2 a, v2 b, v2 c)
    {
        v2 r;
        asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.d) : "l"(a.d), "l"(b.d), "l"(c.d));
        return r;
    }
};

/* (x + L/2) / bin truncated and clamped: the binning rule of the reference's
 * sketch (neighborlist_kernel_o.cu:20-25) with IEEE add and divide. */
/* The coordinate an atom is binned by: its position when every position
 * lies in [-L/2, L/2] (centered), else the periodic image of it in the box.
 * The list predicate measures the positions themselves with the
 * minimum-image shift either way; binning picks only the candidates. */
__device__ __forceinline__ float cell_coord(float x, float L, float Li, int centered)
{
    return centered ? x : __fsub_rn(x, __fmul_rn(L, rintf(__fmul_rn(x, Li))));
}

__device__ __forceinline__ int cell_of(float x, float box, float binlen, int nc)
{
    float s = __fdiv_rn(__fadd_rn(x, box / 2.0f), binlen);
    int c = (s <= 0.0f) ? 0 : (int)s;
    return c >= nc ? nc - 1 : c;
}

/* Asynchronous copies global -> shared (cp.async, sm_80 and later): the
 * data lands while the thread goes on; cp_async_wait() waits for every
 * copy the thread issued.  Both addresses must be aligned to the size, and
 * src must point into global memory. */
__device__ __forceinline__ void cp_async8(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

/* Programmatic dependent launch: a kernel launched with the
 * programmatic-serialization attribute (md_launch_pdl) may be scheduled
 * while its predecessor in the stream still runs.  pdl_wait() blocks until
 * the predecessor has completed and its writes are visible; it returns at
 * once for a kernel launched normally.  pdl_trigger() lets the dependent
 * kernel be scheduled before this kernel's last blocks finish. */
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

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
