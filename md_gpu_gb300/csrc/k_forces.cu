/*
 * k_forces.cu -- pair (LJ + Wolf / reaction field) and bonded forces.
 *
 * Pair forces follow pair_forces.cu:34-205: for each listed j inside rc,
 *   Wolf:  ff = qfac qi qj ([2a/sqrt(pi) r + P5(t) t] e^{-a^2 r^2} / r - W) / r^2,
 *          t = 1/(1 + p a r), P5 = A&S 7.1.26 (simulation.h:39-44),
 *   RF:    ff = qfac qi qj (1/r - k_rf r^2) / r^2,
 *   + LJ:  ff += lj1 r^-14 - lj2 r^-8,
 * F_i += ff d, w_i += ff r^2.  Arithmetic is FP32 (contraction allowed);
 * the per-atom sums are taken in FP32 over chunks of a few neighbours and
 * added into int64 fixed point, so the result does not depend on how the
 * list is split across threads.  TPA lanes share one atom (lane l takes list
 * entries l, l+TPA, ...) and combine with shuffles.
 *
 * Bonded forces follow bonded_forces.cu:34-193 as per-atom gathers over
 * per-atom lists (each bond seen from both atoms, each angle from all three);
 * the centre-atom branch uses the role of the entry being processed.
 */
#include "md_internal.h"

namespace {

#define A1 0.254829592f
#define A2 -0.284496736f
#define A3 1.421413741f
#define A4 -1.453152027f
#define A5 1.061405429f
#define QFAC 1389.35427611722f

struct pair_consts {
    float ucc;     /* Coulomb energy shift at rc */
    float rc6i;    /* rc^-6 */
    float rcinv;   /* 1/rc */
};

/* Round to nearest even for |t| < 2^22 with two FP32 adds (no conversion
 * instruction): the minimum-image shift rint(d / L). */
__device__ __forceinline__ float rint_small(float t)
{
    const float M = 12582912.0f;   /* 1.5 * 2^23 */
    return __fsub_rn(__fadd_rn(t, M), M);
}

/* The hardware approximations (PTX ISA ex2/rsqrt/rcp .approx.ftz): relative
 * errors ~2^-22, well inside the 1e-5 force tolerance; arguments here are
 * never denormal. */
__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

struct pair_acc {
    float fx, fy, fz, fw, fe;
};

/* One pair: F_i += ff d, w_i += ff r^2 (pair_forces.cu:165-200 / :74-120). */
template <int KIND, bool ENERGY>
__device__ __forceinline__ void pair_term(const md_kparams &kp, const pair_consts &pc, float4 pi,
                                          float qi, float4 pj, float2 l, bool valid, pair_acc &a)
{
    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    dx -= kp.box[0] * rint_small(dx * kp.boxi[0]);
    dy -= kp.box[1] * rint_small(dy * kp.boxi[1]);
    dz -= kp.box[2] * rint_small(dz * kp.boxi[2]);
    float rsq = dx * dx + dy * dy + dz * dz;
    float ri = rsqrt_approx(rsq);
    float ri2 = ri * ri;
    float qq = qi * pj.w;
    float ff, uc = 0.0f;
    if (KIND == 1) {
        float r = rsq * ri;
        float t = rcp_approx(1.0f + kp.palfa * r);
        float poly = ((((A5 * t + A4) * t + A3) * t + A2) * t + A1) * t;
        float ex = ex2_approx(kp.alfasq * rsq);
        ff = ((kp.spiialfa * r + poly) * ex * ri - kp.wolf) * qq;
        if (ENERGY) uc = qq * (poly * ex * ri - pc.ucc + kp.wolf * __logf(r * pc.rcinv));
    } else {
        ff = qq * (ri - kp.reacf * rsq);
        if (ENERGY) uc = qq * (ri + 0.5f * kp.reacf * rsq - pc.ucc);
    }
    float ri6 = ri2 * ri2 * ri2;
    ff = ff * ri2 + (l.x * ri6 - l.y) * ri6 * ri2;
    /* list padding entries point at the atom itself: r = 0 is skipped */
    bool in = valid && rsq <= kp.rcutsq && rsq > 0.0f;
    ff = in ? ff : 0.0f;
    a.fx += ff * dx;
    a.fy += ff * dy;
    a.fz += ff * dz;
    a.fw += ff * rsq;
    if (ENERGY) {
        float ulj = l.x * (1.0f / 12.0f) * (ri6 * ri6 - pc.rc6i * pc.rc6i) -
                    l.y * (1.0f / 6.0f) * (ri6 - pc.rc6i);
        a.fe += in ? 0.5f * (uc + ulj) : 0.0f;
    }
}

/* Pair forces of atom i from its list: TPA lanes per atom, lane l takes the
 * entries l, l+TPA, ... in batches of B (TPA*B divides 32, the padding
 * quantum of the list rows, so no entry needs a bounds test).  The loads are
 * software pipelined: while batch t is computed, the positions of batch t+1
 * and the list entries of batch t+2 are in flight.  Each lane sums in FP32
 * and converts its sum to int64 once; lane sums are combined with integer
 * shuffles (exact), so the result depends only on TPA. */
template <int KIND, int TPA, int B, bool ENERGY>
__global__ void __launch_bounds__(128) k_pair(md_kparams kp, pair_consts pc,
                                              const float4 *__restrict__ pos4,
                                              const int *__restrict__ type,
                                              const unsigned *__restrict__ nl,
                                              const int *__restrict__ nl_n,
                                              const float2 *__restrict__ ljtab, long long *f,
                                              float *vir, float *epot)
{
    static_assert(MD_LIST_QUANTUM % (TPA * B) == 0, "batch must divide the list padding");
    __shared__ float2 lj[MD_MAXTYPE * MD_MAXTYPE];
    if (threadIdx.x < MD_MAXTYPE * MD_MAXTYPE) lj[threadIdx.x] = ljtab[threadIdx.x];
    __syncthreads();
    int gt = blockIdx.x * blockDim.x + threadIdx.x;
    int i = gt / TPA, lane = gt % TPA;
    bool active = i < kp.n;
    int ii = active ? i : 0;
    const float4 pi = pos4[ii];
    const int cnt = active ? nl_n[ii] : 0;
    const int nb = ((cnt + MD_LIST_QUANTUM - 1) / MD_LIST_QUANTUM) * (MD_LIST_QUANTUM / (TPA * B));
    const float2 *ljrow = lj + type[ii] * MD_MAXTYPE;
    const float qi = QFAC * pi.w;
    pair_acc acc = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    const unsigned *lp = nl + (size_t)ii * kp.cap + lane;
    unsigned e0[B], e1[B];
    float4 p0[B];
    if (nb > 0) {
#pragma unroll
        for (int b = 0; b < B; b++) e0[b] = __ldg(lp + b * TPA);
#pragma unroll
        for (int b = 0; b < B; b++) p0[b] = __ldg(pos4 + (e0[b] & MD_INDEX_MASK));
    }
    if (nb > 1) {
#pragma unroll
        for (int b = 0; b < B; b++) e1[b] = __ldg(lp + (B + b) * TPA);
    }
#pragma unroll 2
    for (int t = 0; t < nb; t++) {
        float4 p1[B];
        unsigned e2[B];
        if (t + 1 < nb) {
#pragma unroll
            for (int b = 0; b < B; b++) p1[b] = __ldg(pos4 + (e1[b] & MD_INDEX_MASK));
        }
        if (t + 2 < nb) {
#pragma unroll
            for (int b = 0; b < B; b++) e2[b] = __ldg(lp + ((t + 2) * B + b) * TPA);
        }
#pragma unroll
        for (int b = 0; b < B; b++)
            pair_term<KIND, ENERGY>(kp, pc, pi, qi, p0[b], ljrow[e0[b] >> MD_TYPE_SHIFT], true, acc);
#pragma unroll
        for (int b = 0; b < B; b++) {
            e0[b] = e1[b];
            p0[b] = p1[b];
            e1[b] = e2[b];
        }
    }
    long long ax = __float2ll_rn(acc.fx * 4294967296.0f);
    long long ay = __float2ll_rn(acc.fy * 4294967296.0f);
    long long az = __float2ll_rn(acc.fz * 4294967296.0f);
    float fw = acc.fw, fe = acc.fe;
    if (TPA > 1) {
        const unsigned mask = 0xffffffffu;
#pragma unroll
        for (int off = TPA / 2; off > 0; off >>= 1) {
            ax += __shfl_down_sync(mask, ax, off, TPA);
            ay += __shfl_down_sync(mask, ay, off, TPA);
            az += __shfl_down_sync(mask, az, off, TPA);
            fw += __shfl_down_sync(mask, fw, off, TPA);
            if (ENERGY) fe += __shfl_down_sync(mask, fe, off, TPA);
        }
    }
    const size_t P = (size_t)kp.pitch;
    if (active && lane == 0) {
        f[i] = ax;
        f[P + i] = ay;
        f[2 * P + i] = az;
        vir[i] = fw;
        if (ENERGY) epot[i] = fe;
    }
}

__device__ __forceinline__ void min_image(float &dx, float &dy, float &dz, const md_kparams &kp)
{
    dx -= kp.box[0] * rintf(dx * kp.boxi[0]);
    dy -= kp.box[1] * rintf(dy * kp.boxi[1]);
    dz -= kp.box[2] * rintf(dz * kp.boxi[2]);
}

/* Harmonic bonds (U = k (r - r0)^2, bnd1 = 2k) and angles (U = k (th - th0)^2,
 * ang1 = 2k), one thread per sorted atom, added into the fixed-point forces. */
template <bool ENERGY>
__global__ void k_bonded(md_kparams kp, const float4 *__restrict__ pos4,
                         const int2 *__restrict__ bl_s, const int *__restrict__ bl_sn,
                         const int4 *__restrict__ al_s, const int *__restrict__ al_sn,
                         const float *__restrict__ par, int has_bonds, int has_angles,
                         long long *f, float *vir, float *epot)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= kp.n) return;
    const int P = kp.pitch;
    int nb = has_bonds ? bl_sn[s] : 0;
    int na = has_angles ? al_sn[s] : 0;
    if (nb == 0 && na == 0) return;
    const float *bnd1 = par, *bnd2 = par + MD_MAXTYPE, *ang1 = par + 2 * MD_MAXTYPE,
                *ang2 = par + 3 * MD_MAXTYPE;
    float4 p = pos4[s];
    float fx = 0.0f, fy = 0.0f, fz = 0.0f, fw = 0.0f, fe = 0.0f;
    for (int k = 0; k < nb; k++) {
        int2 b = bl_s[k * P + s];
        float4 q = pos4[b.x];
        float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
        min_image(dx, dy, dz, kp);
        float rsq = dx * dx + dy * dy + dz * dz;
        float ri = rsqrtf(rsq);
        float kk = bnd1[b.y], r0 = bnd2[b.y];
        float fa = kk * (r0 * ri - 1.0f);
        fw += fa * rsq;
        fx += fa * dx; fy += fa * dy; fz += fa * dz;
        if (ENERGY) { float dr = rsq * ri - r0; fe += 0.25f * kk * dr * dr; }
    }
    for (int k = 0; k < na; k++) {
        int4 a = al_s[k * P + s];
        float4 qa, qb = pos4[a.z];
        float4 cen;
        if (a.x == 1) { qa = pos4[a.y]; cen = p; }   /* this atom is the centre */
        else { qa = p; cen = pos4[a.y]; }           /* this atom is an end */
        float ax = qa.x - cen.x, ay = qa.y - cen.y, az = qa.z - cen.z;
        min_image(ax, ay, az, kp);
        float bx = qb.x - cen.x, by = qb.y - cen.y, bz = qb.z - cen.z;
        min_image(bx, by, bz, kp);
        float ai = rsqrtf(ax * ax + ay * ay + az * az);
        float bi = rsqrtf(bx * bx + by * by + bz * bz);
        float ab = ax * bx + ay * by + az * bz;
        float cang = ab * ai * bi;
        cang = fminf(fmaxf(cang, -0.9999999f), 0.9999999f);
        float th = acosf(cang);
        float ff = ang1[a.w] * (th - ang2[a.w]) * rsqrtf(1.0f - cang * cang) * ai * bi;
        float aa = ab * ai * ai;
        float gx = bx - aa * ax, gy = by - aa * ay, gz = bz - aa * az;
        if (a.x == 1) {
            float bb = ab * bi * bi;
            gx = bb * bx - ax - gx;
            gy = bb * by - ay - gy;
            gz = bb * bz - az - gz;
        }
        fx += ff * gx; fy += ff * gy; fz += ff * gz;
        if (ENERGY) { float dth = th - ang2[a.w]; fe += 0.5f * ang1[a.w] * dth * dth * (1.0f / 3.0f); }
    }
    f[s] += __float2ll_rn(fx * 4294967296.0f);
    f[P + s] += __float2ll_rn(fy * 4294967296.0f);
    f[2 * P + s] += __float2ll_rn(fz * 4294967296.0f);
    vir[s] += fw;
    if (ENERGY) epot[s] += fe;
}

template <int KIND, bool ENERGY>
void pair_dispatch(md_ctx *c, const md_kparams &kp, const pair_consts &pc)
{
    long long threads = (long long)kp.n * c->pair_tpa;
    int nb = (int)((threads + 127) / 128);
    const float2 *lj = (const float2 *)c->lj_dev;
    switch (c->pair_tpa) {
#define MD_PAIR_CASE(T)                                                                          \
    case T:                                                                                      \
        k_pair<KIND, T, (T >= 32 ? 1 : (T >= 16 ? 2 : (T >= 8 ? 4 : 8))), ENERGY>               \
            <<<nb, 128, 0, c->stream>>>(                                                         \
            kp, pc, c->pos4, c->type, c->nl, c->nl_n, lj, c->f, c->vir, c->epot);                \
        break;
        MD_PAIR_CASE(1)
        MD_PAIR_CASE(2)
        MD_PAIR_CASE(4)
        MD_PAIR_CASE(8)
        MD_PAIR_CASE(16)
        MD_PAIR_CASE(32)
#undef MD_PAIR_CASE
    default:
        break;
    }
}

}  // namespace

void launch_forces(md_ctx *c, const md_kparams &kp, bool energy, int terms)
{
    pair_consts pc;
    double rc = sqrt((double)c->rcutsq);
    pc.rcinv = (float)(1.0 / rc);
    pc.rc6i = (float)(1.0 / (rc * rc * rc * rc * rc * rc));
    if (c->lkspace == 1) {
        double a = c->alfa, x = a * rc;
        double t = 1.0 / (1.0 + (double)0.3275911f * x);
        double poly = ((((double)A5 * t + (double)A4) * t + (double)A3) * t + (double)A2) * t + (double)A1;
        pc.ucc = (float)(poly * t * exp(-x * x) / rc);
    } else if (c->lkspace == 0) {
        pc.ucc = (float)(1.0 / rc + 0.5 * (double)c->reacf * rc * rc);
    } else {
        pc.ucc = 0.0f;
    }
    if (terms & MD_TERM_PAIR) {
        if (c->lkspace == 0) {
            if (energy) pair_dispatch<0, true>(c, kp, pc);
            else pair_dispatch<0, false>(c, kp, pc);
        } else {
            if (energy) pair_dispatch<1, true>(c, kp, pc);
            else pair_dispatch<1, false>(c, kp, pc);
        }
    } else {
        cudaMemsetAsync(c->f, 0, sizeof(long long) * 3 * (size_t)c->pitch, c->stream);
        cudaMemsetAsync(c->vir, 0, sizeof(float) * (size_t)c->pitch, c->stream);
        cudaMemsetAsync(c->epot, 0, sizeof(float) * (size_t)c->pitch, c->stream);
    }
    int hb = (terms & MD_TERM_BOND) ? c->has_bonds : 0;
    int ha = (terms & MD_TERM_ANGLE) ? c->has_angles : 0;
    if (hb || ha) {
        int nb = (kp.n + 255) / 256;
        if (energy)
            k_bonded<true><<<nb, 256, 0, c->stream>>>(kp, c->pos4, c->bl_s, c->bl_sn, c->al_s,
                                                       c->al_sn, c->bonded_par, hb, ha,
                                                       c->f, c->vir, c->epot);
        else
            k_bonded<false><<<nb, 256, 0, c->stream>>>(kp, c->pos4, c->bl_s, c->bl_sn, c->al_s,
                                                        c->al_sn, c->bonded_par, hb, ha,
                                                        c->f, c->vir, c->epot);
    }
}
