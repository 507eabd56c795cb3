/*
 * k_noalloc.cu -- kinetic energy and temperature of a velocity array in the
 * reference's float4 layout, computed without allocating device memory.
 *
 * Some callers cannot let a library call cudaMalloc: hosts that own every
 * byte of device memory through their own allocator and budget (an MD engine
 * or framework embedding this path as a plugin), and step loops that must not
 * risk the device-wide synchronisation cudaMalloc/cudaFree can cause.  For
 * them this file keeps the per-block partial sums of the reduction in a fixed
 * file-scope __device__ array instead of allocated scratch.
 *
 * Limits and rules:
 *  - at most MD_NOALLOC_MAX_ATOMS atoms per call (4096 blocks of 256 threads,
 *    32 KB of scratch); larger calls are rejected with MD_ERR_ARG;
 *  - the array lives on every device that loads the library until the
 *    process exits;
 *  - every call shares it: calls whose kernels overlap on the GPU (different
 *    streams, no ordering between them) race on the partial sums; order them
 *    on one stream or synchronise between them;
 *  - host code cannot use the array's symbol as a pointer: every call made
 *    outside stream capture looks up its device address on the current
 *    device with cudaGetSymbolAddress (cheap, allocates nothing), so an
 *    address cached before a cudaDeviceReset (which loads the module again)
 *    is never used; a call made while its stream is being captured cannot
 *    make that lookup safely and reuses the address the last uncaptured
 *    call on the device resolved, so make one call on each device before
 *    capturing.
 */
#include <mutex>

#include "md_internal.h"

#define MD_NOALLOC_BLOCK 256
#define MD_NOALLOC_MAX_BLOCKS 4096
#define MD_NOALLOC_MAX_ATOMS (MD_NOALLOC_BLOCK * MD_NOALLOC_MAX_BLOCKS)
#define MD_NOALLOC_MAX_DEVICES 64

/* Per-block partial sums of m v^2 / 2; every call overwrites the first
 * ceil(natom/256) entries before reading them, so nothing needs clearing. */
static __device__ __align__(256) double g_ke_partials[MD_NOALLOC_MAX_BLOCKS];

namespace {

constexpr double RGAS = 8.314e-3;   /* kJ/mol/K, as integrator.cu:155 (1000/8.314) */

std::mutex g_mu;
double *g_partials_addr[MD_NOALLOC_MAX_DEVICES] = {};

__device__ __forceinline__ double block_sum256(double v, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < MD_NOALLOC_BLOCK / 32; k++) r += sh[k];
    return r;
}

/* vel4[i] = (vx, vy, vz, m*1e4): per-block sum of m v^2 / 2 in FP64. */
__global__ void __launch_bounds__(MD_NOALLOC_BLOCK) k_ke_partials(const float4 *__restrict__ vel4,
                                                                  int n, double *partials)
{
    __shared__ double sh[MD_NOALLOC_BLOCK / 32];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double ke = 0.0;
    if (i < n) {
        float4 v = vel4[i];
        double vx = v.x, vy = v.y, vz = v.z;
        ke = 0.5 * (double)v.w * (vx * vx + vy * vy + vz * vz);
    }
    double s = block_sum256(ke, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

/* One block: fixed-order sum of the partials; out[0] = KE, out[1] = T. */
__global__ void __launch_bounds__(MD_NOALLOC_BLOCK) k_ke_finish(const double *__restrict__ partials,
                                                                int nblocks, int n, double *out)
{
    __shared__ double sh[MD_NOALLOC_BLOCK / 32];
    double a = 0.0;
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) a += partials[k];
    double ke = block_sum256(a, sh);
    if (threadIdx.x == 0) {
        out[0] = ke;
        out[1] = 2.0 * ke / ((3.0 * n - 3.0) * RGAS);
    }
}

}  // namespace

extern "C" md_status md_ref_kinetic_energy_noalloc(const void *vel4, int natom, double *out,
                                                   void *stream)
{
    if (!vel4 || !out || natom < 2) {
        md_set_global_error("md_ref_kinetic_energy_noalloc: null pointer or fewer than 2 atoms");
        return MD_ERR_ARG;
    }
    if (natom > MD_NOALLOC_MAX_ATOMS) {
        md_set_global_error("md_ref_kinetic_energy_noalloc: natom " + std::to_string(natom) +
                            " exceeds the fixed scratch limit of " +
                            std::to_string(MD_NOALLOC_MAX_ATOMS) + " atoms");
        return MD_ERR_ARG;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= MD_NOALLOC_MAX_DEVICES) {
        md_set_global_error("md_ref_kinetic_energy_noalloc: no usable current device");
        return MD_ERR_CUDA;
    }
    cudaStream_t s = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(s, &cap);
    if (e != cudaSuccess) {
        md_set_global_error(std::string("md_ref_kinetic_energy_noalloc: cudaStreamIsCapturing: ") +
                            cudaGetErrorString(e));
        return MD_ERR_CUDA;
    }
    double *partials = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (cap == cudaStreamCaptureStatusNone) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_ke_partials);
            if (e != cudaSuccess) {
                md_set_global_error(std::string("md_ref_kinetic_energy_noalloc: cudaGetSymbolAddress: ") +
                                    cudaGetErrorString(e));
                return MD_ERR_CUDA;
            }
            g_partials_addr[dev] = (double *)p;
        }
        partials = g_partials_addr[dev];
    }
    if (!partials) {
        md_set_global_error("md_ref_kinetic_energy_noalloc: first call on this device made during stream "
                            "capture; make one call before capturing");
        return MD_ERR_ARG;
    }
    int nb = (natom + MD_NOALLOC_BLOCK - 1) / MD_NOALLOC_BLOCK;
    k_ke_partials<<<nb, MD_NOALLOC_BLOCK, 0, s>>>((const float4 *)vel4, natom, partials);
    k_ke_finish<<<1, MD_NOALLOC_BLOCK, 0, s>>>(partials, nb, natom, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        md_set_global_error(std::string("md_ref_kinetic_energy_noalloc: launch: ") + cudaGetErrorString(e));
        return MD_ERR_CUDA;
    }
    return MD_OK;
}
