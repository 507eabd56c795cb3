/*
 * k_pair64.cu -- the FP64 mode of the force kernels (md_set_precision(ctx,
 * 64)): the same pair and bonded force laws as the FP32 kernels, evaluated
 * in FP64 on the FP64 positions, with IEEE sqrt, divide, exp and log.
 *
 * This is the "plain FP64" form of the path run on the GPU: the reference
 * point of the precision gates (RMS force error, NVE drift) and the per-system
 * FP64 runs the adjoint's throughput is compared with.  The force law follows
 * pair_forces.cu:34-205 with the reference's A&S 7.1.26 erfc
 * (simulation.h:39-44, its float coefficients widened to FP64) and Wolf
 * shift W = rc Ft(rc) (forces.cu:104-110); bonds and angles follow
 * bonded_forces.cu:34-193 (U = k (r - r0)^2 with bnd1 = 2k, U = k (th -
 * th0)^2 with ang1 = 2k).  Forces go into the same int64 fixed-point arrays
 * (2^-32 kJ/mol/A: the rounding, ~1e-10 kJ/mol/A, is far below FP32's), so
 * the integrators, thermostats and reductions are shared with the FP32 mode.
 *
 * Layout: 8 lanes per atom, 16 atoms per block of 128 threads; lane l takes
 * the list entries l, l+8, ... of its atom's padded row (the padding entries
 * point at the atom itself, r = 0, and are skipped); each lane sums in FP64,
 * rounds its sums to fixed point once, and the lanes combine with integer
 * shuffles, so the result is deterministic.
 */
#include <cstddef>
#include <cstring>

#include "md_pair.cuh"

namespace {

constexpr int P64_TPA = 8;
constexpr int P64_THREADS = 128;
constexpr int P64_ATOMS = P64_THREADS / P64_TPA;

/* One pair: ff (F_i = ff d) and the pair energy (consistent potential,
 * LJ shifted to zero at rc) for r^2 <= rc^2. */
template <int KIND, bool ENERGY>
__device__ __forceinline__ void pair64_eval(const md_p64 &m, double rsq, double qq, double lja,
                                            double ljc, double &ff, double &u)
{
    const double r = sqrt(rsq), ri = 1.0 / r, ri2 = ri * ri;
    double fc, uc = 0.0;
    if (KIND == 1) {
        const double xa = m.alpha * r;
        const double t = 1.0 / (1.0 + m.pex * xa);
        const double p = ((((m.a[4] * t + m.a[3]) * t + m.a[2]) * t + m.a[1]) * t + m.a[0]);
        const double ex = exp(-xa * xa);
        const double ec = p * t * ex;
        fc = qq * ((ec * ri + m.spi * ex) - m.wolfw) * ri2;
        if (ENERGY) uc = qq * (ec * ri - m.ucc + m.wolfw * log(r * m.rcinv));
    } else {
        fc = qq * (ri * ri2 - m.reacf);
        if (ENERGY) uc = qq * (ri + 0.5 * m.reacf * rsq - m.ucc);
    }
    const double ri6 = ri2 * ri2 * ri2, ri8 = ri6 * ri2;
    ff = fc + (lja * ri6 * ri8 - ljc * ri8);
    if (ENERGY)
        u = uc + (lja * (1.0 / 12.0) * (ri6 * ri6 - m.rc6i * m.rc6i) - ljc * (1.0 / 6.0) * (ri6 - m.rc6i));
}

/* Pair forces in FP64 of a single system (tab == nullptr: block b holds
 * atoms 16b .. 16b+15) or of a batch (block b holds up to 16 atoms of
 * replica tab[b].x from tab[b].y on; geometry, model and LJ table per
 * replica). */
template <int KIND, bool ENERGY>
__global__ void __launch_bounds__(P64_THREADS) k_pair64(int n, int pitch, int cap, int centered,
                                                       const int2 *__restrict__ tab,
                                                       const md_rep *__restrict__ reps,
                                                       const md_p64 *__restrict__ models,
                                                       const float2 *__restrict__ ljtab,
                                                       const double *__restrict__ x,
                                                       const float4 *__restrict__ pos4,
                                                       const int *__restrict__ type,
                                                       const unsigned *__restrict__ nl,
                                                       const int *__restrict__ nl_n, long long *f,
                                                       float *vir, float *epot)
{
    __shared__ double2 lj[MD_MAXTYPE * MD_MAXTYPE];
    pdl_trigger();   /* the integrator may be scheduled; it waits for this grid */
    int rep = 0, i0, end;
    if (tab) {
        const int2 bt = tab[blockIdx.x];
        rep = bt.x;
        i0 = bt.y;
        end = reps[rep].atom0 + reps[rep].natom;
    } else {
        i0 = blockIdx.x * P64_ATOMS;
        end = n;
    }
    const md_p64 m = models[rep];
    if (threadIdx.x < MD_MAXTYPE * MD_MAXTYPE) {
        const float2 l = ljtab[(size_t)rep * MD_MAXTYPE * MD_MAXTYPE + threadIdx.x];
        lj[threadIdx.x] = make_double2((double)l.x, (double)l.y);
    }
    __syncthreads();
    const int i = i0 + (int)threadIdx.x / P64_TPA, lane = (int)threadIdx.x % P64_TPA;
    const bool active = i < end;
    const int ii = active ? i : i0;
    const size_t P = (size_t)pitch;
    const double xi = x[ii], yi = x[P + ii], zi = x[2 * P + ii];
    const double qi = m.qfac * (double)pos4[ii].w;
    const double2 *ljrow = lj + type[ii] * MD_MAXTYPE;
    const int cnt = active ? nl_n[ii] : 0;
    const int npad = (cnt + P64_TPA - 1) / P64_TPA * P64_TPA;   /* padding past it adds zero */
    /* a warp whose atoms all lie at least rc from every face (positions
     * centred in the box) needs no minimum-image shift for any pair inside
     * rc: the shift is L * 0 there, and a pair beyond L/2 is beyond rc */
    const bool in_i = fabs(xi) + m.rc < 0.499 * m.L[0] && fabs(yi) + m.rc < 0.499 * m.L[1] &&
                      fabs(zi) + m.rc < 0.499 * m.L[2];
    const bool inner = centered && __all_sync(0xffffffffu, !active || in_i);
    double fx = 0.0, fy = 0.0, fz = 0.0, fw = 0.0, fe = 0.0;
    const unsigned *row = nl + (size_t)ii * cap;
    for (int k = lane; k < npad; k += P64_TPA) {
        const unsigned e = __ldg(row + k);
        const int j = (int)(e & MD_INDEX_MASK);
        double dx = xi - x[j], dy = yi - x[P + j], dz = zi - x[2 * P + j];
        if (!inner) {
            dx -= m.L[0] * rint(dx * m.Li[0]);
            dy -= m.L[1] * rint(dy * m.Li[1]);
            dz -= m.L[2] * rint(dz * m.Li[2]);
        }
        const double rsq = dx * dx + dy * dy + dz * dz;
        if (rsq <= m.rcsq && rsq > 0.0) {
            const double2 l = ljrow[e >> MD_TYPE_SHIFT];
            double ff, u = 0.0;
            pair64_eval<KIND, ENERGY>(m, rsq, qi * (double)pos4[j].w, l.x, l.y, ff, u);
            fx += ff * dx;
            fy += ff * dy;
            fz += ff * dz;
            fw += ff * rsq;
            if (ENERGY) fe += 0.5 * u;
        }
    }
    long long ix = __double2ll_rn(fx * FX_SCALE), iy = __double2ll_rn(fy * FX_SCALE),
              iz = __double2ll_rn(fz * FX_SCALE);
#pragma unroll
    for (int off = P64_TPA / 2; off > 0; off >>= 1) {
        ix += __shfl_down_sync(0xffffffffu, ix, off, P64_TPA);
        iy += __shfl_down_sync(0xffffffffu, iy, off, P64_TPA);
        iz += __shfl_down_sync(0xffffffffu, iz, off, P64_TPA);
        fw += __shfl_down_sync(0xffffffffu, fw, off, P64_TPA);
        if (ENERGY) fe += __shfl_down_sync(0xffffffffu, fe, off, P64_TPA);
    }
    if (active && lane == 0) {
        f[i] = ix;
        f[P + i] = iy;
        f[2 * P + i] = iz;
        vir[i] = (float)fw;
        if (ENERGY) epot[i] = (float)fe;
    }
}

/* Harmonic bonds and angles in FP64 on the FP64 positions, one thread per
 * sorted atom (each bond seen from both atoms, each angle from all three),
 * added into the fixed-point forces; the same formulas as k_bonded.  In a
 * batch (reps non-null) the minimum image uses the atom's replica box. */
template <bool ENERGY>
__global__ void k_bonded64(int n, int pitch, const double *__restrict__ boxd,
                           const double *__restrict__ x, const int2 *__restrict__ bl_s,
                           const int *__restrict__ bl_sn, const int4 *__restrict__ al_s,
                           const int *__restrict__ al_sn, const float *__restrict__ par, int has_bonds,
                           int has_angles, const md_rep *__restrict__ reps, const int *__restrict__ arep,
                           long long *f, float *vir, float *epot)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const size_t P = (size_t)pitch;
    const int nb = has_bonds ? bl_sn[s] : 0;
    const int na = has_angles ? al_sn[s] : 0;
    if (nb == 0 && na == 0) return;
    const double *L = reps ? reps[arep[s]].boxd : boxd;
    const double Li[3] = {1.0 / L[0], 1.0 / L[1], 1.0 / L[2]};
    const float *bnd1 = par, *bnd2 = par + MD_MAXTYPE, *ang1 = par + 2 * MD_MAXTYPE,
                *ang2 = par + 3 * MD_MAXTYPE;
    auto pos = [&](int a, double *o) {
        o[0] = x[a];
        o[1] = x[P + a];
        o[2] = x[2 * P + a];
    };
    auto diff = [&](const double *a, const double *b, double *d) {
        for (int k = 0; k < 3; k++) {
            d[k] = a[k] - b[k];
            d[k] -= L[k] * rint(d[k] * Li[k]);
        }
    };
    double p[3];
    pos(s, p);
    double fx = 0.0, fy = 0.0, fz = 0.0, fw = 0.0, fe = 0.0;
    for (int k = 0; k < nb; k++) {
        const int2 b = bl_s[k * P + s];
        double q[3], d[3];
        pos(b.x, q);
        diff(p, q, d);
        const double rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const double r = sqrt(rsq);
        const double kk = bnd1[b.y], r0 = bnd2[b.y];
        const double fa = kk * (r0 / r - 1.0);
        fw += fa * rsq;
        fx += fa * d[0];
        fy += fa * d[1];
        fz += fa * d[2];
        if (ENERGY) {
            const double dr = r - r0;
            fe += 0.25 * kk * dr * dr;
        }
    }
    for (int k = 0; k < na; k++) {
        const int4 a = al_s[k * P + s];
        double qa[3], qb[3], cen[3], va[3], vb[3];
        pos(a.z, qb);
        if (a.x == 1) {   /* this atom is the centre */
            pos(a.y, qa);
            cen[0] = p[0]; cen[1] = p[1]; cen[2] = p[2];
        } else {          /* this atom is an end */
            qa[0] = p[0]; qa[1] = p[1]; qa[2] = p[2];
            pos(a.y, cen);
        }
        diff(qa, cen, va);
        diff(qb, cen, vb);
        const double ai = 1.0 / sqrt(va[0] * va[0] + va[1] * va[1] + va[2] * va[2]);
        const double bi = 1.0 / sqrt(vb[0] * vb[0] + vb[1] * vb[1] + vb[2] * vb[2]);
        const double ab = va[0] * vb[0] + va[1] * vb[1] + va[2] * vb[2];
        double cang = ab * ai * bi;
        cang = fmin(fmax(cang, -0.9999999), 0.9999999);
        const double th = acos(cang);
        const double ff = (double)ang1[a.w] * (th - (double)ang2[a.w]) / sqrt(1.0 - cang * cang) * ai * bi;
        const double aa = ab * ai * ai;
        double g[3] = {vb[0] - aa * va[0], vb[1] - aa * va[1], vb[2] - aa * va[2]};
        if (a.x == 1) {
            const double bb = ab * bi * bi;
            for (int q = 0; q < 3; q++) g[q] = bb * vb[q] - va[q] - g[q];
        }
        fx += ff * g[0];
        fy += ff * g[1];
        fz += ff * g[2];
        if (ENERGY) {
            const double dth = th - (double)ang2[a.w];
            fe += 0.5 * (double)ang1[a.w] * dth * dth * (1.0 / 3.0);
        }
    }
    f[s] += __double2ll_rn(fx * FX_SCALE);
    f[P + s] += __double2ll_rn(fy * FX_SCALE);
    f[2 * P + s] += __double2ll_rn(fz * FX_SCALE);
    vir[s] += (float)fw;
    if (ENERGY) epot[s] += (float)fe;
}

}  // namespace

/* FP64 model constants of one system (pairmodel of the plain form): rc from
 * the FP32 rc^2 as given, the Wolf shift and energy constants with the A&S
 * erfc in FP64. */
md_p64 md_make_p64(int lkspace, float rcutsq, float reacf, float alfa, const float box[3])
{
    md_p64 m;
    memset(&m, 0, sizeof(m));
    m.kind = lkspace;
    m.rcsq = (double)rcutsq;
    m.rc = sqrt(m.rcsq);
    m.rcinv = 1.0 / m.rc;
    const double rc2i = 1.0 / m.rcsq;
    m.rc6i = rc2i * rc2i * rc2i;
    m.reacf = lkspace == 0 ? (double)reacf : 0.0;
    m.alpha = (double)alfa;
    m.spi = 2.0 / sqrt(3.14159265358979323846) * m.alpha;
    m.pex = (double)0.3275911f;
    m.a[0] = (double)A1;
    m.a[1] = (double)A2;
    m.a[2] = (double)A3;
    m.a[3] = (double)A4;
    m.a[4] = (double)A5;
    m.qfac = (double)QFAC;
    for (int k = 0; k < 3; k++) {
        m.L[k] = (double)box[k];
        m.Li[k] = 1.0 / m.L[k];
    }
    if (lkspace == 1) {
        const double xa = m.alpha * m.rc;
        const double t = 1.0 / (1.0 + m.pex * xa);
        const double p = ((((m.a[4] * t + m.a[3]) * t + m.a[2]) * t + m.a[1]) * t + m.a[0]);
        const double ec = p * t * exp(-xa * xa);
        m.wolfw = ec / m.rc + m.spi * exp(-m.alpha * m.alpha * m.rcsq);
        m.ucc = ec / m.rc;
    } else if (lkspace == 0) {
        m.ucc = 1.0 / m.rc + 0.5 * m.reacf * m.rcsq;
    }
    return m;
}

void launch_pair64(md_ctx *c, bool energy)
{
    const bool batch = c->batch != 0;
    const int2 *tab = nullptr;
    int nb;
    if (batch) {
        const int k = md_grid_index(P64_ATOMS);
        tab = c->grid_tab + c->grid_off[k];
        nb = c->grid_cnt[k];
    } else {
        nb = (c->n + P64_ATOMS - 1) / P64_ATOMS;
    }
    const float2 *lj = batch ? c->ljr_dev : (const float2 *)c->lj_dev;
    const md_rep *reps = batch ? c->reps_dev : nullptr;
#define MD_P64_ARGS                                                                                \
    c->n, c->pitch, c->cap, c->centered, tab, reps, (const md_p64 *)c->p64_dev, lj, (const double *)c->x, \
        (const float4 *)c->pos4, (const int *)c->type, (const unsigned *)c->nl, (const int *)c->nl_n, c->f, \
        c->vir, c->epot
    if (c->lkspace == 0) {
        if (energy) k_pair64<0, true><<<nb, P64_THREADS, 0, c->stream>>>(MD_P64_ARGS);
        else k_pair64<0, false><<<nb, P64_THREADS, 0, c->stream>>>(MD_P64_ARGS);
    } else {
        if (energy) k_pair64<1, true><<<nb, P64_THREADS, 0, c->stream>>>(MD_P64_ARGS);
        else k_pair64<1, false><<<nb, P64_THREADS, 0, c->stream>>>(MD_P64_ARGS);
    }
#undef MD_P64_ARGS
}

void launch_bonded64(md_ctx *c, bool energy, int hb, int ha)
{
    const int nb = (c->n + 255) / 256;
    const md_rep *reps = c->batch ? c->reps_dev : nullptr;
    const int *arep = c->batch ? c->arep : nullptr;
    /* a single system: the box of model 0 (a device address; not read here) */
    const double *boxd = (const double *)((const char *)c->p64_dev + offsetof(md_p64, L));
    if (energy)
        k_bonded64<true><<<nb, 256, 0, c->stream>>>(c->n, c->pitch, boxd, c->x, c->bl_s, c->bl_sn, c->al_s,
                                                    c->al_sn, c->bonded_par, hb, ha, reps, arep, c->f,
                                                    c->vir, c->epot);
    else
        k_bonded64<false><<<nb, 256, 0, c->stream>>>(c->n, c->pitch, boxd, c->x, c->bl_s, c->bl_sn, c->al_s,
                                                     c->al_sn, c->bonded_par, hb, ha, reps, arep, c->f,
                                                     c->vir, c->epot);
}
