/*
 * k_integrate.cu -- integrators and the FP64 thermodynamic reductions.
 *
 * Leapfrog (nve_leapfrog.cu:31-60, nvt_leapfrog_ber.cu:29-80):
 *   v <- (v + F dt/m') lambda,  x <- x + v dt,  x -= L trunc(2x/L)
 * with lambda = sqrt(1 + dt/tau (T0/T_prev - 1)) for Berendsen NVT
 * (integrator.cu:146-147, tau = 100 fs there) and 1 for NVE.  Positions and
 * velocities are FP64 here; the FP32 copy pos4 is refreshed in the same pass.
 * The kinetic energy of every (atom, axis) is FP64 and is summed exactly in
 * fixed point (2^-24 kJ/mol; integer shuffles, one atomic add per block),
 * replacing the reference's single-block FP32 tree (nvt_leapfrog_ber.cu:
 * 83-110, whose width is the block count).
 *
 * The same pass performs the next step's neighbour-list check (any atom moved
 * >= skin/2 since the last build, neighborlist.cu:157-176) and, inside a
 * captured step graph, sets the condition of the rebuild node that follows.
 *
 * Velocity Verlet: half kick + drift (+ list check), forces, half kick.
 * Nose-Hoover adds a thermostat half step on each side (one thermostat,
 * Trotter splitting):
 *   xi += G dt/4;  v *= exp(-xi dt/2);  eta += xi dt/2;  xi += G dt/4,
 *   G = (2 KE - ndf k T0) / Q,  Q = ndf k T0 tau^2,
 * with the conserved quantity KE + PE + Q xi^2/2 + ndf k T0 eta.
 */
#include <algorithm>

#include "md_thermo.cuh"

namespace {

/* The integrators run one thread per (atom, axis): MD_LA atoms per block,
 * axis = threadIdx.x / MD_LA, so each axis streams a contiguous run of the
 * SoA arrays and the FP64 chains of one atom run in three threads (the FP64
 * pipe is slow and deep here: more independent chains hide its latency).
 * The new FP32 positions meet in shared memory, where one thread per atom
 * writes pos4 and performs the list check.
 *
 * Leapfrog update + list check + KE sums; the last block finalises.
 * kick[s] = dt/m * 2^-32 turns the fixed-point force into the velocity
 * change directly (the same product as F dt/m, rounded once). */
__global__ void __launch_bounds__(3 * MD_LA) k_leapfrog(md_kparams kp, thermo_par tp, step_io io,
                                                       double *x, double *v,
                                                       const double *__restrict__ mass,
                                                       const double *__restrict__ kick,
                                                       float4 *pos4,
                                                       const long long *__restrict__ f,
                                                       const float *__restrict__ epot,
                                                       const float *__restrict__ vir)
{
    __shared__ long long sh[3 * (3 * MD_LA / 32)];
    __shared__ float s_x[3][MD_LA];
    pdl_wait();      /* the forces of this step */
    pdl_trigger();   /* the list passes that follow may be scheduled */
    const int d = threadIdx.x / MD_LA, a = threadIdx.x - d * MD_LA;
    const int s = blockIdx.x * MD_LA + a;
    const size_t o = (size_t)d * kp.pitch + s;
    long long ke = 0, pe = 0, w = 0;
    if (s < kp.n) {
        const axis_par ax = axis_of(d, kp.wlim, kp.boxd, kp.box2i);
        double vv = v[o] + (double)f[o] * kick[s];
        if (tp.berendsen) vv *= io.st->lam_next;
        v[o] = vv;
        double xx = x[o] + vv * kp.dt;
        s_x[d][a] = wrap(xx, ax.lim, ax.L, ax.two_over_l);
        x[o] = xx;
        ke = ke_fix(mass[s], vv);
        if (d == 0 && tp.energy) {
            pe = llrint((double)epot[s] * MD_EFIX);
            w = llrint((double)vir[s] * MD_EFIX);
        }
    }
    __syncthreads();
    bool moved = false;
    if (d == 0 && s < kp.n) {
        float4 p = make_float4(s_x[0][a], s_x[1][a], s_x[2][a], pos4[s].w);
        pos4[s] = p;
        moved = md_rsq_exact(p, io.pos_old[s], kp) >= kp.rmaxdif;
    }
    if (block_close(ke, pe, w, tp.energy ? 3 : 1, moved, io.st, io.counter, sh)) {
        finalize(kp, tp, 0, io.st, io.rec, io.rec_cap);
        set_condition(io);
        *io.counter = 0;
    }
}

/* Velocity Verlet first half: thermostat half step (NH), half kick, drift,
 * list check; the last block sets the rebuild condition. */
__global__ void __launch_bounds__(3 * MD_LA) k_vv_first(md_kparams kp, thermo_par tp, step_io io,
                                                       double *x, double *v,
                                                       const double *__restrict__ kick,
                                                       float4 *pos4,
                                                       const long long *__restrict__ f)
{
    __shared__ float s_x[3][MD_LA];
    __shared__ long long sh[3 * (3 * MD_LA / 32)];
    pdl_trigger();   /* the list passes that follow may be scheduled */
    const int d = threadIdx.x / MD_LA, a = threadIdx.x - d * MD_LA;
    const int s = blockIdx.x * MD_LA + a;
    const size_t o = (size_t)d * kp.pitch + s;
    md_devstate *st = io.st;
    /* pending thermostat factor and, for NH, the first half step of this
     * step, both prepared by the previous step's reduction */
    const double scale = st->kick_scale;
    if (s < kp.n) {
        const axis_par ax = axis_of(d, kp.wlim, kp.boxd, kp.box2i);
        double vv = v[o];
        if (scale != 1.0) vv *= scale;
        vv += (double)f[o] * (0.5 * kick[s]);
        v[o] = vv;
        double xx = x[o] + vv * kp.dt;
        s_x[d][a] = wrap(xx, ax.lim, ax.L, ax.two_over_l);
        x[o] = xx;
    }
    __syncthreads();
    bool moved = false;
    if (d == 0 && s < kp.n) {
        float4 p = make_float4(s_x[0][a], s_x[1][a], s_x[2][a], pos4[s].w);
        pos4[s] = p;
        moved = md_rsq_exact(p, io.pos_old[s], kp) >= kp.rmaxdif;
    }
    if (block_close(0, 0, 0, 0, moved, st, io.counter, sh)) {
        set_condition(io);
        *io.counter = 0;
    }
}

/* Velocity Verlet second half kick and KE (PE, virial) sums; the last
 * block finalises.  do_kick = 0: observe the state only (pending NH scale
 * applied), mode 2. */
__global__ void __launch_bounds__(3 * MD_LA) k_vv_second(md_kparams kp, thermo_par tp, int do_kick,
                                                        step_io io, double *v,
                                                        const double *__restrict__ mass,
                                                        const double *__restrict__ kick,
                                                        const long long *__restrict__ f,
                                                        const float *__restrict__ epot,
                                                        const float *__restrict__ vir)
{
    __shared__ long long sh[3 * (3 * MD_LA / 32)];
    pdl_wait();   /* the forces of this step */
    const int d = threadIdx.x / MD_LA, a = threadIdx.x - d * MD_LA;
    const int s = blockIdx.x * MD_LA + a;
    const size_t o = (size_t)d * kp.pitch + s;
    long long ke = 0, pe = 0, w = 0;
    if (s < kp.n) {
        double vv = v[o];
        if (do_kick) {
            vv += (double)f[o] * (0.5 * kick[s]);
            v[o] = vv;
        } else {
            vv *= io.st->vscale;
        }
        ke = ke_fix(mass[s], vv);
        if (d == 0 && tp.energy) {
            pe = llrint((double)epot[s] * MD_EFIX);
            w = llrint((double)vir[s] * MD_EFIX);
        }
    }
    if (block_close(ke, pe, w, tp.energy ? 3 : 1, false, io.st, io.counter, sh)) {
        finalize(kp, tp, do_kick ? 1 : 2, io.st, io.rec, io.rec_cap);
        *io.counter = 0;
    }
}

/* Original-order output: what 0 positions (3), 1 velocities (3, pending NH
 * scale applied), 2 forces + sum ff r^2 (4), 3 per-atom energy (1),
 * 4 velocities as stored (3, pending scale not applied). */
__global__ void k_gather_out(md_kparams kp, int what, const md_devstate *st,
                             const md_repstate *__restrict__ repst, const int *__restrict__ arep,
                             const int *__restrict__ perm, const double *__restrict__ x,
                             const double *__restrict__ v, const long long *__restrict__ f,
                             const float *__restrict__ vir, const float *__restrict__ epot,
                             double *out)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= kp.n) return;
    const int P = kp.pitch;
    int o = perm[s];
    if (what == 0) {
        for (int d = 0; d < 3; d++) out[3 * (size_t)o + d] = x[d * P + s];
    } else if (what == 1) {
        double sc = repst ? repst[arep[s]].vscale : st->vscale;
        for (int d = 0; d < 3; d++) out[3 * (size_t)o + d] = v[d * P + s] * sc;
    } else if (what == 4) {
        for (int d = 0; d < 3; d++) out[3 * (size_t)o + d] = v[d * P + s];
    } else if (what == 2) {
        for (int d = 0; d < 3; d++) out[4 * (size_t)o + d] = (double)f[d * P + s] * FX_INV;
        out[4 * (size_t)o + 3] = vir[s];
    } else {
        out[o] = epot[s];
    }
}

/* Original-order input: what 0 positions (also refreshes pos4), 1 velocities. */
__global__ void k_scatter_in(md_kparams kp, int what, md_devstate *st, md_repstate *repst,
                             int nrep, const int *__restrict__ iperm, const double *__restrict__ in,
                             double *x, double *v, float4 *pos4)
{
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o == 0 && what == 1) st->vscale = 1.0;
    if (repst && o < nrep && what == 1) repst[o].vscale = 1.0;
    if (o >= kp.n) return;
    const int P = kp.pitch;
    int s = iperm[o];
    if (what == 0) {
        double xn[3];
        for (int d = 0; d < 3; d++) {
            xn[d] = in[3 * (size_t)o + d];
            x[d * P + s] = xn[d];
        }
        float4 p = pos4[s];
        pos4[s] = make_float4((float)xn[0], (float)xn[1], (float)xn[2], p.w);
    } else {
        for (int d = 0; d < 3; d++) v[d * P + s] = in[3 * (size_t)o + d];
    }
}

}  // namespace

void launch_leapfrog(md_ctx *c, const md_kparams &kp, int energy, unsigned long long cond, int has_cond)
{
    if (c->batch) {
        launch_leapfrog_b(c, kp, energy, cond, has_cond);
        return;
    }

    int nb = (kp.n + MD_LA - 1) / MD_LA;
    md_launch_pdl(k_leapfrog, dim3(nb), dim3(3 * MD_LA), c->stream, kp, make_tp(c, energy),
                  make_io(c, cond, has_cond), c->x, c->v, (const double *)c->mass,
                  (const double *)c->kick, c->pos4, (const long long *)c->f,
                  (const float *)c->epot, (const float *)c->vir);
}

void launch_vv_first(md_ctx *c, const md_kparams &kp, unsigned long long cond, int has_cond)
{
    if (c->batch) {
        launch_vv_first_b(c, kp, cond, has_cond);
        return;
    }

    int nb = (kp.n + MD_LA - 1) / MD_LA;
    k_vv_first<<<nb, 3 * MD_LA, 0, c->stream>>>(kp, make_tp(c, 0), make_io(c, cond, has_cond), c->x,
                                          c->v, c->kick, c->pos4, c->f);
}

void launch_vv_second(md_ctx *c, const md_kparams &kp, int energy)
{
    if (c->batch) {
        launch_vv_second_b(c, kp, energy, 1);
        return;
    }

    int nb = (kp.n + MD_LA - 1) / MD_LA;
    md_launch_pdl(k_vv_second, dim3(nb), dim3(3 * MD_LA), c->stream, kp, make_tp(c, energy), 1,
                  make_io(c, 0, 0), c->v, (const double *)c->mass, (const double *)c->kick,
                  (const long long *)c->f, (const float *)c->epot, (const float *)c->vir);
}

void launch_thermo_from_state(md_ctx *c, const md_kparams &kp, int energy)
{
    if (c->batch) {
        launch_vv_second_b(c, kp, energy, 0);
        return;
    }

    int nb = (kp.n + MD_LA - 1) / MD_LA;
    k_vv_second<<<nb, 3 * MD_LA, 0, c->stream>>>(kp, make_tp(c, energy), 0, make_io(c, 0, 0), c->v,
                                           c->mass, c->kick, c->f, c->epot, c->vir);
}

void launch_gather_out(md_ctx *c, const md_kparams &kp, int what, void *dst)
{
    int nb = (kp.n + 255) / 256;
    k_gather_out<<<nb, 256, 0, c->stream>>>(kp, what, c->st, c->batch ? c->repst : nullptr,
                                            c->arep, c->perm, c->x, c->v, c->f, c->vir, c->epot,
                                            (double *)dst);
}

void launch_scatter_in(md_ctx *c, const md_kparams &kp, int what, const void *src)
{
    int nb = (kp.n + 255) / 256;
    int nbs = std::max(nb, (c->nrep + 255) / 256);
    k_scatter_in<<<nbs, 256, 0, c->stream>>>(kp, what, c->st, c->batch ? c->repst : nullptr,
                                             c->nrep, c->iperm, (const double *)src, c->x, c->v,
                                             c->pos4);
}
