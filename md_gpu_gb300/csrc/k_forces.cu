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
#include "md_pair.cuh"

namespace {

/* The pair forces of atom ii (see pair_sum) written to the force arrays. */
template <int KIND, int TPA, int B, bool ENERGY>
__global__ void __launch_bounds__(128) k_pair(md_kparams kp, pair_consts pc,
                                              const float4 *__restrict__ pos4,
                                              const int *__restrict__ type,
                                              const unsigned *__restrict__ nl,
                                              const int *__restrict__ nl_n,
                                              const float2 *__restrict__ ljtab, long long *f,
                                              float *vir, float *epot)
{
    __shared__ float2 lj[MD_MAXTYPE * MD_MAXTYPE];
    pdl_trigger();   /* the integrator may be scheduled; it waits for this grid */
    if (threadIdx.x < MD_MAXTYPE * MD_MAXTYPE) lj[threadIdx.x] = ljtab[threadIdx.x];
    __syncthreads();
    int gt = blockIdx.x * blockDim.x + threadIdx.x;
    int i = gt / TPA, lane = gt % TPA;
    bool active = i < kp.n;
    pair_total t = pair_sum<KIND, TPA, B, ENERGY>(geom_kp{kp, pc}, kp.cap, active ? i : 0, active, lane, pos4, type,
                                                  nl, nl_n, lj);
    const size_t P = (size_t)kp.pitch;
    if (active && lane == 0) {
        f[i] = t.fx;
        f[P + i] = t.fy;
        f[2 * P + i] = t.fz;
        vir[i] = t.fw;
        if (ENERGY) epot[i] = t.fe;
    }
}

__device__ __forceinline__ void min_image(float &dx, float &dy, float &dz, const float *box, const float *boxi)
{
    dx -= box[0] * rintf(dx * boxi[0]);
    dy -= box[1] * rintf(dy * boxi[1]);
    dz -= box[2] * rintf(dz * boxi[2]);
}

/* Harmonic bonds (U = k (r - r0)^2, bnd1 = 2k) and angles (U = k (th - th0)^2,
 * ang1 = 2k), one thread per sorted atom, added into the fixed-point forces.
 * In a batch (reps non-null) the minimum image uses the atom's replica box. */
template <bool ENERGY>
__global__ void k_bonded(md_kparams kp, const float4 *__restrict__ pos4,
                         const int2 *__restrict__ bl_s, const int *__restrict__ bl_sn,
                         const int4 *__restrict__ al_s, const int *__restrict__ al_sn,
                         const float *__restrict__ par, int has_bonds, int has_angles,
                         const md_rep *__restrict__ reps, const int *__restrict__ arep,
                         long long *f, float *vir, float *epot)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= kp.n) return;
    const int P = kp.pitch;
    int nb = has_bonds ? bl_sn[s] : 0;
    int na = has_angles ? al_sn[s] : 0;
    if (nb == 0 && na == 0) return;
    const float *box = reps ? reps[arep[s]].box : kp.box, *boxi = reps ? reps[arep[s]].boxi : kp.boxi;
    const float *bnd1 = par, *bnd2 = par + MD_MAXTYPE, *ang1 = par + 2 * MD_MAXTYPE,
                *ang2 = par + 3 * MD_MAXTYPE;
    float4 p = pos4[s];
    float fx = 0.0f, fy = 0.0f, fz = 0.0f, fw = 0.0f, fe = 0.0f;
    for (int k = 0; k < nb; k++) {
        int2 b = bl_s[k * P + s];
        float4 q = pos4[b.x];
        float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
        min_image(dx, dy, dz, box, boxi);
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
        min_image(ax, ay, az, box, boxi);
        float bx = qb.x - cen.x, by = qb.y - cen.y, bz = qb.z - cen.z;
        min_image(bx, by, bz, box, boxi);
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
    const int key = c->pair_tpa * 100 + md_pair_depth(c);
    switch (key) {
#define MD_PAIR_CASE(T, BB)                                                                      \
    case T * 100 + BB:                                                                           \
        k_pair<KIND, T, BB, ENERGY><<<nb, 128, 0, c->stream>>>(                                  \
            kp, pc, c->pos4, c->type, c->nl, c->nl_n, lj, c->f, c->vir, c->epot);                \
        break;
        MD_PAIR_CASE(1, 8)
        MD_PAIR_CASE(2, 8)
        MD_PAIR_CASE(4, 4)
        MD_PAIR_CASE(4, 8)
        MD_PAIR_CASE(8, 2)
        MD_PAIR_CASE(8, 4)
        MD_PAIR_CASE(16, 1)
        MD_PAIR_CASE(16, 2)
        MD_PAIR_CASE(32, 1)
#undef MD_PAIR_CASE
    default:
        break;
    }
}

}  // namespace

void launch_forces(md_ctx *c, const md_kparams &kp, bool energy, int terms)
{
    if (c->batch) {
        launch_forces_b(c, kp, energy, terms);
        return;
    }
    pair_consts pc = make_pair_consts(c);
    if ((terms & MD_TERM_PAIR) && c->fp64) {
        launch_pair64(c, energy);
    } else if (terms & MD_TERM_PAIR) {
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
    launch_bonded(c, kp, energy, terms);
    if (c->pme.on && (terms & MD_TERM_RECIP)) launch_pme(c, kp, energy);
}

void launch_bonded(md_ctx *c, const md_kparams &kp, bool energy, int terms)
{
    int hb = (terms & MD_TERM_BOND) ? c->has_bonds : 0;
    int ha = (terms & MD_TERM_ANGLE) ? c->has_angles : 0;
    if ((hb || ha) && c->fp64) {
        launch_bonded64(c, energy, hb, ha);
    } else if (hb || ha) {
        int nb = (kp.n + 255) / 256;
        const md_rep *reps = c->batch ? c->reps_dev : nullptr;
        const int *arep = c->batch ? c->arep : nullptr;
        if (energy)
            k_bonded<true><<<nb, 256, 0, c->stream>>>(kp, c->pos4, c->bl_s, c->bl_sn, c->al_s,
                                                       c->al_sn, c->bonded_par, hb, ha, reps, arep,
                                                       c->f, c->vir, c->epot);
        else
            k_bonded<false><<<nb, 256, 0, c->stream>>>(kp, c->pos4, c->bl_s, c->bl_sn, c->al_s,
                                                        c->al_sn, c->bonded_par, hb, ha, reps, arep,
                                                        c->f, c->vir, c->epot);
    }
}
