/*
 * k_pme.cu -- the reciprocal-space part of the Ewald sum by smooth
 * particle-mesh Ewald (SPME, Essmann et al., J. Chem. Phys. 103, 8577
 * (1995)) with cubic B-splines, for lkspace 2 ("Ewald", whose real-space
 * term the pair kernels compute: simulation.cu:91-95, forces.cu:97-113).
 * The reference carries SPME only as an unbuilt copy of GROMACS's pme.c
 * (make_bsplines :1222, make_bspline_moduli :1297, spread_q_bsplines :829,
 * solve_pme :941, gather_f_bsplines :1136); this is the same method built
 * for one GPU:
 *
 *   prep    one thread per atom: spline origin, offsets and charge;
 *   spread  one block per 8^3 brick of the charge grid gathers the charges
 *           of the atoms whose splines reach it, found through the cell
 *           lists; sums in 2^-32 fixed point in shared memory, as two
 *           32-bit parts (order independent, so the grid is the same bit
 *           for bit every run; a 2^-20 grid in one 32-bit sum measured
 *           3.8e-5 RMS relative force error on NaCl, where Na and Cl
 *           weights cancel on the grid), each grid point written once, no
 *           global atomics;
 *   FFT     cuFFT, real to complex, FP32;
 *   solve   the half spectrum times B(m) C(m) (a table made on the host);
 *   FFT     complex to real: the convolution theta_rec * Q on the grid;
 *   gather  one thread per atom: potential and its gradient from the 64
 *           grid points of its splines; forces added into the int64
 *           fixed-point forces, energies into the per-atom energies (with
 *           the self term and the share of a net charge's background);
 *   excl    one thread per atom: removes the excluded partners' erf(a r)/r
 *           term that the reciprocal sum holds (the pair list omits them).
 *
 * Grid convention: u_d = K_d frac((x_d + L_d/2) (1/L_d)), i0 = floor(u),
 * w = u - i0; the points i0 - 3 .. i0 (periodic) carry M4(w + 3 - j).
 */
#include <cufft.h>

#include <algorithm>

#include "md_device.cuh"
#include "md_internal.h"

namespace {

constexpr int PB = 8;                 /* brick edge, grid points */
constexpr int PW = PB + 3;            /* window of spline origins i0 that reach a brick */
constexpr int PME_MAXC = 8;           /* candidate cells per axis of a brick */
constexpr float QSCALE = 4294967296.0f;  /* 2^32: fixed point of the spread grid */
constexpr double QFAC_D = 1389.35427611722;

struct pme_par {
    int K[3];
    double L[3], Li[3];   /* box and 1/L */
    float kl[3];       /* K / L */
    float h[3];        /* L / K */
    int nc[3];
    float binlen[3];
    float margin;      /* how far an atom may have left its cell since the last build */
    int ncand[3];      /* candidate cells per axis (<= PME_MAXC, <= nc) */
    int n;
    int pitch;
    float self_c;      /* QFAC alpha / sqrt(pi) */
    float e_bg;        /* background energy of a net charge, per atom */
};

/* Spline origin and fractional offset of one coordinate (the library's
 * convention; 1/L as a multiplication: FP64 division is a long sequence on
 * this GPU's FP64 pipe). */
__device__ __forceinline__ int spline_origin(double x, double L, double Li, int K, float &w)
{
    double t = (x + 0.5 * L) * Li;
    t -= floor(t);
    const double u = (double)K * t;
    const double f = floor(u);
    w = (float)(u - f);
    int i0 = (int)f;
    if (i0 >= K) i0 -= K;
    /* a non-finite coordinate (a run that has blown up) must not index
     * outside the grid */
    return min(max(i0, 0), K - 1);
}

__device__ __forceinline__ void bspline4(float w, float th[4])
{
    const float v = 1.0f - w, w2 = w * w, w3 = w2 * w;
    th[0] = v * v * v * (1.0f / 6.0f);
    th[1] = (3.0f * w3 - 6.0f * w2 + 4.0f) * (1.0f / 6.0f);
    th[2] = (-3.0f * w3 + 3.0f * w2 + 3.0f * w + 1.0f) * (1.0f / 6.0f);
    th[3] = w3 * (1.0f / 6.0f);
}

__device__ __forceinline__ void bspline4_d(float w, float dt[4])
{
    const float v = 1.0f - w, w2 = w * w;
    dt[0] = -0.5f * v * v;
    dt[1] = 0.5f * (3.0f * w2 - 4.0f * w);
    dt[2] = 0.5f * (-3.0f * w2 + 2.0f * w + 1.0f);
    dt[3] = 0.5f * w2;
}

/* Per atom, once per force evaluation: spline origins (x, y, z) and the
 * offsets and charge (w_x, w_y, w_z, q), read by the spread (for every
 * brick an atom's cell is a candidate of) and by the gather. */
__global__ void k_pme_prep(pme_par pp, const double *__restrict__ x, const float4 *__restrict__ pos4,
                           int4 *__restrict__ org, float4 *__restrict__ wq)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= pp.n) return;
    float w[3];
    int i0[3];
    for (int d = 0; d < 3; d++)
        i0[d] = spline_origin(x[(size_t)d * pp.pitch + s], pp.L[d], pp.Li[d], pp.K[d], w[d]);
    org[s] = make_int4(i0[0], i0[1], i0[2], 0);
    wq[s] = make_float4(w[0], w[1], w[2], pos4[s].w);
}

/* Charge grid, one block per brick (see the file comment).  The block
 * walks the candidate atoms 256 at a time: each thread tests one and
 * queues it (spline origin relative to the brick, its 12 weights, charge)
 * when its spline reaches the brick; then the block's threads take the
 * queued atoms' 64 (atom, point) products one each, so every lane adds one
 * grid point per pass instead of one thread looping over an atom's 64. */
__global__ void __launch_bounds__(256) k_pme_spread(pme_par pp, const int4 *__restrict__ org,
                                                    const float4 *__restrict__ wq,
                                                    const int *__restrict__ cell_rank,
                                                    const int *__restrict__ cell_start, float *grid)
{
    /* the 2^-32 fixed-point sum of a grid point as two 32-bit sums (native
     * shared-memory atomics): v = hi 2^20 + lo with lo = v mod 2^20; lo
     * sums stay exact for up to 2048 contributions per point, hi for
     * charges below 256 e */
    __shared__ int s_hi[PB * PB * PB];
    __shared__ int s_lo[PB * PB * PB];
    __shared__ int s_start[PME_MAXC * PME_MAXC * PME_MAXC];   /* first atom of each candidate cell */
    __shared__ int s_pre[PME_MAXC * PME_MAXC * PME_MAXC + 1];
    __shared__ int s_rel[256];          /* queued atom: (rx, ry, rz) packed 8 bits each */
    __shared__ float s_th[256][13];     /* queued atom: x, y, z weights (4 each) and charge */
    __shared__ int s_nq;
    const int tid = threadIdx.x;
    const int nbz = pp.K[2] / PB, nby = pp.K[1] / PB;
    const int bz = blockIdx.x % nbz, by = (blockIdx.x / nbz) % nby, bx = blockIdx.x / (nbz * nby);
    const int lo[3] = {bx * PB, by * PB, bz * PB};
    for (int t = tid; t < PB * PB * PB; t += blockDim.x) {
        s_hi[t] = 0;
        s_lo[t] = 0;
    }
    /* the cells that can hold an atom whose spline origin lies in
     * [lo, lo + PW) on every axis: the grid window in the coordinate
     * x + L/2, widened by the distance an atom may have moved since the
     * cells were filled */
    int first[3];
    for (int d = 0; d < 3; d++) {
        const float a = (float)lo[d] * pp.h[d] - pp.margin;
        first[d] = pp.ncand[d] >= pp.nc[d] ? 0 : (int)floorf(a / pp.binlen[d]);
    }
    const int nca = pp.ncand[0] * pp.ncand[1] * pp.ncand[2];
    if (tid < 32) {
        /* warp 0: ranks and a prefix sum of the candidate cells' atoms */
        int run = 0;
        for (int k0 = 0; k0 < nca; k0 += 32) {
            const int k = k0 + tid;
            int cnt = 0;
            if (k < nca) {
                const int cz = k % pp.ncand[2], cy = (k / pp.ncand[2]) % pp.ncand[1],
                          cx = k / (pp.ncand[2] * pp.ncand[1]);
                int c3[3] = {first[0] + cx, first[1] + cy, first[2] + cz};
                for (int d = 0; d < 3; d++) {
                    c3[d] %= pp.nc[d];
                    if (c3[d] < 0) c3[d] += pp.nc[d];
                }
                const int r = cell_rank[c3[0] + pp.nc[0] * (c3[1] + pp.nc[1] * c3[2])];
                const int b = cell_start[r];
                s_start[k] = b;
                cnt = cell_start[r + 1] - b;
            }
            int incl = cnt;
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (tid >= o) incl += v;
            }
            if (k < nca) s_pre[k] = run + incl - cnt;
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (tid == 0) s_pre[nca] = run;
    }
    __syncthreads();
    const int total = s_pre[nca];
    for (int g0 = 0; g0 < total; g0 += blockDim.x) {
        if (tid == 0) s_nq = 0;
        __syncthreads();
        const int g = g0 + tid;
        if (g < total) {
            /* the candidate cell: the largest k with s_pre[k] <= g */
            int lo_k = 0, hi_k = nca;
            while (hi_k - lo_k > 1) {
                const int m = (lo_k + hi_k) >> 1;
                if (s_pre[m] <= g) lo_k = m; else hi_k = m;
            }
            const int s = s_start[lo_k] + (g - s_pre[lo_k]);
            const int4 o = org[s];
            const float4 a = wq[s];
            int r[3] = {o.x - lo[0], o.y - lo[1], o.z - lo[2]};
            bool in = true;
            for (int d = 0; d < 3; d++) {
                if (r[d] < 0) r[d] += pp.K[d];
                in = in && r[d] < PW;
            }
            if (in && a.w != 0.0f) {
                const int slot = atomicAdd(&s_nq, 1);   /* integer sums: the order is free */
                s_rel[slot] = r[0] | (r[1] << 8) | (r[2] << 16);
                bspline4(a.x, &s_th[slot][0]);
                bspline4(a.y, &s_th[slot][4]);
                bspline4(a.z, &s_th[slot][8]);
                s_th[slot][12] = a.w;
            }
        }
        __syncthreads();
        /* one (atom, x point, y point) row of 4 z points per item */
        const int nw = s_nq * 16;
        for (int t = tid; t < nw; t += blockDim.x) {
            const int at = t >> 4, j = (t >> 2) & 3, k = t & 3;
            const int rl = s_rel[at];
            const int px = (rl & 255) - 3 + j, py = ((rl >> 8) & 255) - 3 + k, pz0 = (rl >> 16) - 3;
            if (px < 0 || px >= PB || py < 0 || py >= PB) continue;
            const float vxy = s_th[at][12] * s_th[at][j] * s_th[at][4 + k];
            const int row = (px * PB + py) * PB;
#pragma unroll
            for (int l = 0; l < 4; l++) {
                const int pz = pz0 + l;
                if (pz < 0 || pz >= PB) continue;
                const long long iv = __float2ll_rn(vxy * s_th[at][8 + l] * QSCALE);
                atomicAdd(&s_hi[row + pz], (int)(iv >> 20));
                atomicAdd(&s_lo[row + pz], (int)(iv & 0xFFFFF));
            }
        }
        __syncthreads();
    }
    for (int t = tid; t < PB * PB * PB; t += blockDim.x) {
        const int px = t / (PB * PB), py = (t / PB) % PB, pz = t % PB;
        grid[((size_t)(lo[0] + px) * pp.K[1] + (lo[1] + py)) * pp.K[2] + (lo[2] + pz)] =
            fmaf((float)s_lo[t], 1.0f / QSCALE, (float)s_hi[t] * (1048576.0f / QSCALE));
    }
}

/* The half spectrum times B(m) C(m). */
__global__ void k_pme_solve(float2 *__restrict__ spec, const float *__restrict__ infl, size_t count)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        const float b = infl[i];
        float2 v = spec[i];
        v.x *= b;
        v.y *= b;
        spec[i] = v;
    }
}

/* Forces and energies of the reciprocal sum from the convolution grid. */
template <bool ENERGY>
__global__ void __launch_bounds__(128) k_pme_gather(pme_par pp, const int4 *__restrict__ org,
                                                    const float4 *__restrict__ wq,
                                                    const float *__restrict__ conv, long long *f,
                                                    float *epot)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= pp.n) return;
    const float4 a = wq[s];
    const float q = a.w;
    if (q == 0.0f) {
        if (ENERGY) epot[s] += pp.e_bg;
        return;
    }
    const int4 o = org[s];
    const float w[3] = {a.x, a.y, a.z};
    const int i0[3] = {o.x, o.y, o.z};
    float tx[4], ty[4], tz[4], dx[4], dy[4], dz[4];
    bspline4(w[0], tx);
    bspline4(w[1], ty);
    bspline4(w[2], tz);
    bspline4_d(w[0], dx);
    bspline4_d(w[1], dy);
    bspline4_d(w[2], dz);
    int iy[4], iz[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        int a = i0[1] - 3 + j, b = i0[2] - 3 + j;
        iy[j] = a < 0 ? a + pp.K[1] : a;
        iz[j] = b < 0 ? b + pp.K[2] : b;
    }
    float phi = 0.0f, gx = 0.0f, gy = 0.0f, gz = 0.0f;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        int a = i0[0] - 3 + j;
        if (a < 0) a += pp.K[0];
        const float *row = conv + (size_t)a * pp.K[1] * pp.K[2];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float *col = row + (size_t)iy[k] * pp.K[2];
            float sv = 0.0f, sd = 0.0f;   /* sums over z with the weight and its derivative */
#pragma unroll
            for (int l = 0; l < 4; l++) {
                const float v = col[iz[l]];
                sv = fmaf(tz[l], v, sv);
                sd = fmaf(dz[l], v, sd);
            }
            phi = fmaf(tx[j] * ty[k], sv, phi);
            gx = fmaf(dx[j] * ty[k], sv, gx);
            gy = fmaf(tx[j] * dy[k], sv, gy);
            gz = fmaf(tx[j] * ty[k], sd, gz);
        }
    }
    const float c = -(float)QFAC_D * q;
    const size_t P = (size_t)pp.pitch;
    f[s] += __float2ll_rn(c * pp.kl[0] * gx * 4294967296.0f);
    f[P + s] += __float2ll_rn(c * pp.kl[1] * gy * 4294967296.0f);
    f[2 * P + s] += __float2ll_rn(c * pp.kl[2] * gz * 4294967296.0f);
    if (ENERGY) epot[s] += 0.5f * (float)QFAC_D * q * phi - pp.self_c * q * q + pp.e_bg;
}

/* Excluded partners of atom s (its own exclusion slots, as its list row
 * omits them): -QFAC q_s q_j erf(a r) / r, force on s only, half the
 * energy. */
template <bool ENERGY>
__global__ void k_pme_excl(md_kparams kp, float alpha, const float4 *__restrict__ pos4,
                           const uint4 *__restrict__ excl_s, long long *f, float *epot)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= kp.n) return;
    const uint4 ex = excl_s[s];
    const unsigned js[4] = {ex.x, ex.y, ex.z, ex.w};
    const float4 p = pos4[s];
    float fx = 0.0f, fy = 0.0f, fz = 0.0f, e = 0.0f;
    const float spi = 1.1283791670955126f * alpha;   /* 2 alpha / sqrt(pi) */
    for (int k = 0; k < 4; k++) {
        if (js[k] == MD_EXCL_NONE) continue;
        const float4 o = pos4[js[k]];
        float dx = p.x - o.x, dy = p.y - o.y, dz = p.z - o.z;
        dx -= kp.box[0] * rintf(dx * kp.boxi[0]);
        dy -= kp.box[1] * rintf(dy * kp.boxi[1]);
        dz -= kp.box[2] * rintf(dz * kp.boxi[2]);
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (r2 <= 0.0f) continue;
        const float r = sqrtf(r2);
        const float qq = (float)QFAC_D * p.w * o.w;
        const float er = erff(alpha * r);
        const float fr = qq * (spi * expf(-alpha * alpha * r2) * r - er) / (r2 * r);
        fx += fr * dx;
        fy += fr * dy;
        fz += fr * dz;
        e -= 0.5f * qq * er / r;
    }
    const size_t P = (size_t)kp.pitch;
    f[s] += __float2ll_rn(fx * 4294967296.0f);
    f[P + s] += __float2ll_rn(fy * 4294967296.0f);
    f[2 * P + s] += __float2ll_rn(fz * 4294967296.0f);
    if (ENERGY) epot[s] += e;
}

/* How far an atom may have moved from the cell it was binned into: less
 * than half the skin (the rebuild criterion), with room for FP32 rounding. */
inline float pme_margin(const md_ctx *c) { return 0.5f * c->skin * 1.001f + 1e-3f; }

pme_par make_pme_par(const md_ctx *c)
{
    pme_par pp;
    for (int d = 0; d < 3; d++) {
        pp.K[d] = c->pme.K[d];
        pp.L[d] = (double)c->box[d];
        pp.Li[d] = 1.0 / pp.L[d];
        pp.kl[d] = (float)((double)pp.K[d] / pp.L[d]);
        pp.h[d] = (float)(pp.L[d] / (double)pp.K[d]);
        pp.nc[d] = c->ncell[d];
        pp.binlen[d] = c->binlen[d];
        pp.ncand[d] = c->pme.ncand[d];
    }
    pp.margin = pme_margin(c);
    pp.n = c->n;
    pp.pitch = c->pitch;
    pp.self_c = (float)(QFAC_D * (double)c->alfa / sqrt(M_PI));
    pp.e_bg = c->pme.e_bg;
    return pp;
}

}  // namespace

static md_status pme_fail(md_ctx *c, md_status s, const std::string &msg)
{
    c->last_error = msg;
    md_set_global_error(msg);
    return s;
}

/* Candidate cells per axis of a brick: the window of PW grid points plus
 * twice the margin, over the cell side, plus one for a window that starts
 * inside a cell.  The window gets 0.01 A of slack, so that the FP32 window
 * the kernel computes never spans one cell more than counted here (a cell
 * too many only adds candidates that fail the test). */
static int pme_cells_per_axis(double L, int K, float binlen, int nc, float margin)
{
    const double win = PW * L / K + 2.0 * margin + 0.01;
    const int n = (int)floor(win / binlen) + 2;
    return std::min(n, nc);
}

md_status pme_setup(md_ctx *c, const int K[3])
{
    pme_free(c);
    if (K[0] == 0 && K[1] == 0 && K[2] == 0) return MD_OK;
    const float margin = pme_margin(c);
    for (int d = 0; d < 3; d++) {
        c->pme.K[d] = K[d];
        c->pme.ncand[d] = pme_cells_per_axis(c->box[d], K[d], c->binlen[d], c->ncell[d], margin);
        if (c->pme.ncand[d] > PME_MAXC) {
            pme_free(c);
            return pme_fail(c, MD_ERR_UNSUPPORTED, "md_set_pme: grid too coarse for the cell grid (more than 8 "
                                                "cells per axis reach one 8-point brick)");
        }
    }
    const size_t nreal = (size_t)K[0] * K[1] * K[2];
    const size_t nspec = (size_t)K[0] * K[1] * (K[2] / 2 + 1);
    MD_CUDA_TRY(c, cudaMalloc(&c->pme.grid, sizeof(float) * nreal));
    MD_CUDA_TRY(c, cudaMalloc(&c->pme.spec, sizeof(float2) * nspec));
    MD_CUDA_TRY(c, cudaMalloc(&c->pme.infl, sizeof(float) * nspec));
    MD_CUDA_TRY(c, cudaMalloc(&c->pme.org, sizeof(int4) * (size_t)c->pitch));
    MD_CUDA_TRY(c, cudaMalloc(&c->pme.wq, sizeof(float4) * (size_t)c->pitch));
    /* B(m) C(m) on the half spectrum, in FP64 on the host */
    std::vector<float> h(nspec);
    const double a = (double)c->alfa;
    const double V = (double)c->box[0] * c->box[1] * c->box[2];
    std::vector<double> mod[3], mm[3];
    for (int d = 0; d < 3; d++) {
        const int len = d == 2 ? K[2] / 2 + 1 : K[d];
        mod[d].resize(len);
        mm[d].resize(len);
        for (int i = 0; i < len; i++) {
            const int m = (d == 2 || i < (K[d] + 1) / 2) ? i : i - K[d];
            const double cs = (2.0 + cos(2.0 * M_PI * m / K[d])) / 3.0;
            mod[d][i] = cs * cs;
            mm[d][i] = m / (double)c->box[d];
        }
    }
    for (int i = 0; i < K[0]; i++)
        for (int j = 0; j < K[1]; j++)
            for (int k = 0; k <= K[2] / 2; k++) {
                const double m2 = mm[0][i] * mm[0][i] + mm[1][j] * mm[1][j] + mm[2][k] * mm[2][k];
                double v = 0.0;
                if (i || j || k)
                    v = exp(-M_PI * M_PI * m2 / (a * a)) / (M_PI * V * m2 * mod[0][i] * mod[1][j] * mod[2][k]);
                h[((size_t)i * K[1] + j) * (K[2] / 2 + 1) + k] = (float)v;
            }
    MD_CUDA_TRY(c, cudaMemcpy(c->pme.infl, h.data(), sizeof(float) * nspec, cudaMemcpyHostToDevice));
    /* the neutralising background of a net charge, shared out per atom */
    double qt = 0.0;
    for (int i = 0; i < c->n; i++) qt += (double)c->charge[i];
    c->pme.e_bg = c->n > 0 ? (float)(-QFAC_D * M_PI * qt * qt / (2.0 * V * a * a) / c->n) : 0.0f;
    c->pme.excl = c->has_bonds ? 1 : 0;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    c->pme.nsm = std::max(1, nsm);
    cufftHandle fwd = 0, inv = 0;
    if (cufftPlan3d(&fwd, K[0], K[1], K[2], CUFFT_R2C) != CUFFT_SUCCESS) {
        pme_free(c);
        return pme_fail(c, MD_ERR_CUDA, "md_set_pme: cufftPlan3d (R2C) failed");
    }
    c->pme.fwd = (int)fwd;
    c->pme.plans = 1;
    if (cufftPlan3d(&inv, K[0], K[1], K[2], CUFFT_C2R) != CUFFT_SUCCESS) {
        pme_free(c);
        return pme_fail(c, MD_ERR_CUDA, "md_set_pme: cufftPlan3d (C2R) failed");
    }
    c->pme.inv = (int)inv;
    c->pme.plans = 2;
    if (cufftSetStream(fwd, c->stream) != CUFFT_SUCCESS || cufftSetStream(inv, c->stream) != CUFFT_SUCCESS) {
        pme_free(c);
        return pme_fail(c, MD_ERR_CUDA, "md_set_pme: cufftSetStream failed");
    }
    c->pme.on = 1;
    return MD_OK;
}

void pme_free(md_ctx *c)
{
    if (c->pme.plans >= 1) cufftDestroy((cufftHandle)c->pme.fwd);
    if (c->pme.plans >= 2) cufftDestroy((cufftHandle)c->pme.inv);
    cudaFree(c->pme.grid);
    cudaFree(c->pme.spec);
    cudaFree(c->pme.infl);
    cudaFree(c->pme.org);
    cudaFree(c->pme.wq);
    c->pme = md_pme();
}

void launch_pme(md_ctx *c, const md_kparams &kp, bool energy)
{
    const pme_par pp = make_pme_par(c);
    const int nbrick = (pp.K[0] / PB) * (pp.K[1] / PB) * (pp.K[2] / PB);
    k_pme_prep<<<(kp.n + 255) / 256, 256, 0, c->stream>>>(pp, c->x, c->pos4, c->pme.org, c->pme.wq);
    k_pme_spread<<<nbrick, 256, 0, c->stream>>>(pp, c->pme.org, c->pme.wq, c->cell_rank, c->cell_start,
                                                c->pme.grid);
    cufftExecR2C((cufftHandle)c->pme.fwd, c->pme.grid, (cufftComplex *)c->pme.spec);
    const size_t nspec = (size_t)pp.K[0] * pp.K[1] * (pp.K[2] / 2 + 1);
    const int sb = (int)std::min<size_t>((nspec + 255) / 256, (size_t)c->pme.nsm * 8);
    k_pme_solve<<<sb, 256, 0, c->stream>>>((float2 *)c->pme.spec, c->pme.infl, nspec);
    cufftExecC2R((cufftHandle)c->pme.inv, (cufftComplex *)c->pme.spec, c->pme.grid);
    const int nb = (kp.n + 127) / 128;
    if (energy)
        k_pme_gather<true><<<nb, 128, 0, c->stream>>>(pp, c->pme.org, c->pme.wq, c->pme.grid, c->f, c->epot);
    else
        k_pme_gather<false><<<nb, 128, 0, c->stream>>>(pp, c->pme.org, c->pme.wq, c->pme.grid, c->f, c->epot);
    if (c->pme.excl) {
        const int ne = (kp.n + 255) / 256;
        if (energy)
            k_pme_excl<true><<<ne, 256, 0, c->stream>>>(kp, c->alfa, c->pos4, c->excl_s, c->f, c->epot);
        else
            k_pme_excl<false><<<ne, 256, 0, c->stream>>>(kp, c->alfa, c->pos4, c->excl_s, c->f, c->epot);
    }
}
