/*
 * k_probe.cu -- measurement helpers: the pair kernel timed on its own, and
 * an FP32 FMA throughput probe that gives the measured FP32-pipe peak the
 * pair kernel's roofline is quoted against.
 */
#include "md_internal.h"

namespace {

/* Eight independent FMA chains per thread; the result is kept live through a
 * data-dependent store that never fires for the inputs used. */
__global__ void __launch_bounds__(256) k_fma_probe(float *out, int iters, float a, float b)
{
    float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.0f, x2 = x0 + 2.0f, x3 = x0 + 3.0f;
    float x4 = x0 + 4.0f, x5 = x0 + 5.0f, x6 = x0 + 6.0f, x7 = x0 + 7.0f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < 8; u++) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == -1.2345e30f) out[blockIdx.x] = s;
}

}  // namespace

extern "C" md_status md_time_pair(md_ctx *c, int nrep, float *ms_per_launch)
{
    if (!c || nrep <= 0 || !ms_per_launch) return MD_ERR_ARG;
    md_kparams kp = md_make_kparams(c);
    launch_forces(c, kp, false, MD_TERM_PAIR);   /* warm */
    MD_CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
    for (int r = 0; r < nrep; r++) launch_forces(c, kp, false, MD_TERM_PAIR);
    MD_CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    MD_CUDA_TRY(c, cudaEventSynchronize(c->ev1));
    float ms = 0.0f;
    MD_CUDA_TRY(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    *ms_per_launch = ms / nrep;
    /* the last evaluation leaves only pair forces: restore the full force */
    launch_forces(c, kp, false, MD_TERM_ALL);
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MD_OK;
}

extern "C" md_status md_time_rebuild(md_ctx *c, int nrep, float *ms_per_build)
{
    if (!c || nrep <= 0 || !ms_per_build) return MD_ERR_ARG;
    md_kparams kp = md_make_kparams(c);
    launch_rebuild(c, kp, true, true);   /* warm */
    MD_CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
    for (int r = 0; r < nrep; r++) launch_rebuild(c, kp, true, true);
    MD_CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    MD_CUDA_TRY(c, cudaEventSynchronize(c->ev1));
    float ms = 0.0f;
    MD_CUDA_TRY(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    *ms_per_build = ms / nrep;
    /* positions did not change: forces of the re-sorted state are recomputed */
    launch_forces(c, kp, false, MD_TERM_ALL);
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MD_OK;
}

extern "C" md_status md_probe_fp32_peak(double *tflops)
{
    if (!tflops) return MD_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MD_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return MD_ERR_CUDA;
    float *out = nullptr;
    cudaEvent_t e0, e1;
    if (cudaMalloc(&out, sizeof(float) * 65536) != cudaSuccess) return MD_ERR_CUDA;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    k_fma_probe<<<blocks, threads>>>(out, 64, 1.0000001f, 1e-7f);   /* warm */
    float best = 1e30f;
    for (int r = 0; r < 5; r++) {
        cudaEventRecord(e0);
        k_fma_probe<<<blocks, threads>>>(out, iters, 1.0000001f, 1e-7f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return MD_ERR_CUDA;
    double flops = 2.0 * 64.0 * iters * (double)threads * blocks;
    *tflops = flops / (best * 1e-3) / 1e12;
    return MD_OK;
}
