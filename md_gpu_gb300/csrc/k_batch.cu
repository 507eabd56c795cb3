/*
 * k_batch.cu -- pair forces and integrators of a batch of independent
 * replicas (md_create_batch), each with its own box, cutoffs, LJ table and
 * charges, advanced together by one launch per stage.
 *
 * The replicas' atoms are concatenated; a replica's atoms stay one
 * contiguous range through every re-sort.  Every launch here runs on a
 * replica-aligned grid (md_rep, grid_tab): a block covers atoms of one
 * replica only, so the replica's geometry and force-field constants are
 * uniform across the block (kept in registers, its LJ table in shared
 * memory), and each block adds its energy sums into its replica's
 * fixed-point accumulators.  The arithmetic per atom is the single-system arithmetic
 * (pair_sum, the leapfrog / velocity-Verlet updates of k_integrate.cu), so a
 * replica advances bit-for-bit as it would alone with the same tuning.
 */
#include "md_pair.cuh"
#include "md_thermo.cuh"

namespace {

/* Pair forces of a batch: block b holds 128/TPA atoms of replica tab[b].x
 * starting at tab[b].y. */
template <int KIND, int TPA, int B, bool ENERGY>
__global__ void __launch_bounds__(128) k_pair_b(int cap, int pitch, int centered,
                                                const int2 *__restrict__ tab,
                                                const md_rep *__restrict__ reps,
                                                const float2 *__restrict__ ljr,
                                                const float4 *__restrict__ pos4,
                                                const int *__restrict__ type,
                                                const unsigned *__restrict__ nl,
                                                const int *__restrict__ nl_n, long long *f,
                                                float *vir, float *epot)
{
    __shared__ float2 lj[MD_MAXTYPE * MD_MAXTYPE];
    pdl_trigger();   /* the integrator may be scheduled; it waits for this grid */
    const int2 bt = tab[blockIdx.x];
    const md_rep &R = reps[bt.x];
    if (threadIdx.x < MD_MAXTYPE * MD_MAXTYPE)
        lj[threadIdx.x] = ljr[bt.x * MD_MAXTYPE * MD_MAXTYPE + threadIdx.x];
    const geom_reg g = rep_geom(R, centered != 0);
    const int end = R.atom0 + R.natom;
    __syncthreads();
    const int i = bt.y + (int)threadIdx.x / TPA, lane = (int)threadIdx.x % TPA;
    const bool active = i < end;
    /* unrolled twice: measured faster here than rolled (1.46 against 1.56 ms
     * per launch on the 512-replica batch) */
    pair_total t = pair_sum<KIND, TPA, B, ENERGY, true, 2>(g, cap, active ? i : bt.y, active, lane, pos4,
                                                  type, nl, nl_n, lj);
    const size_t P = (size_t)pitch;
    if (active && lane == 0) {
        f[i] = t.fx;
        f[P + i] = t.fy;
        f[2 * P + i] = t.fz;
        vir[i] = t.fw;
        if (ENERGY) epot[i] = t.fe;
    }
}

/* Runs in the last block to finish: one thread per replica turns its
 * accumulators into KE, PE and virial (and clears them for the next step),
 * then does the replica's thermostat bookkeeping; the batch's step record
 * sums the replicas in a fixed order. */
__device__ void finalize_b(const md_kparams &kp, const thermo_par &tp, int mode, int nrep,
                           const md_rep *__restrict__ reps, md_repstate *repst,
                           unsigned long long *racc, md_devstate *st, md_thermo *rec, int rec_cap,
                           double *rep_hist, double *sh)
{
    double tke = 0.0, tpe = 0.0, tw = 0.0, tex = 0.0;
    /* the step this record belongs to (thread 0 advances it after the sums) */
    const long long step = ((volatile md_devstate *)st)->step;
    const int builds = ((volatile md_devstate *)st)->builds;
    double *hist = (rep_hist && mode != 2) ? rep_hist + (size_t)(step & (rec_cap - 1)) * 3 * nrep : nullptr;
    for (int r = threadIdx.x; r < nrep; r += blockDim.x) {
        const md_rep &R = reps[r];
        const double a = fix_take(racc + 3 * r, MD_KFIX);
        double b = fix_take(racc + 3 * r + 1, MD_EFIX);
        double c = fix_take(racc + 3 * r + 2, MD_EFIX);
        if (tp.npt && mode == 0) {
            /* P = (2 KE + sum_pairs F.r) / (3 V); c = sum over atoms of ff r^2,
             * every pair counted from both atoms; V of the box the forces saw */
            const double V = R.boxd[0] * R.boxd[1] * R.boxd[2];
            const double P = (2.0 * a + 0.5 * c) / (3.0 * V);
            double mu = 1.0 - R.mu_k * (R.p0 - P);
            mu = fmin(fmax(mu, 1.0 - R.mu_max), 1.0 + R.mu_max);
            repst[r].pressure = P;
            repst[r].mu_used = repst[r].mu_next;
            repst[r].mu_next = mu;
        }
        if (!tp.energy) b = c = 0.0;
        thermo_par t = tp;
        t.t0 = R.t0;
        t.ndf = R.ndf;
        t.q_nh = R.q_nh;
        t.inv_ndfr = R.inv_ndfr;
        t.inv_q = R.inv_q;
        double xi, eta, lam;
        double ke = thermo_advance(kp.dt, t, mode, a, b, c, repst + r, &xi, &eta, &lam);
        tke += ke;
        tpe += b;
        tw += c;
        const double ex = t.nh ? 0.5 * t.q_nh * xi * xi + t.ndf * RGAS * t.t0 * eta : 0.0;
        tex += ex;
        if (hist) {
            hist[3 * r] = ke;
            hist[3 * r + 1] = tp.energy ? b : 0.0;
            hist[3 * r + 2] = tp.energy ? ke + b + ex : 0.0;
        }
    }
    const double KE = block_sum(tke, sh);
    const double PE = block_sum(tpe, sh);
    const double W = block_sum(tw, sh);
    const double EX = block_sum(tex, sh);
    if (threadIdx.x != 0) return;
    st->ke = KE;
    if (tp.energy) {
        st->pe = PE;
        st->virial = W / 6.0;
    }
    if (mode == 2) return;
    st->temper = 2.0 * KE * tp.inv_ndfr;
    write_record(tp, tp.inv_ndfr, KE, PE, W, EX, 0.0, 1.0, step, builds, st, rec, rec_cap);
}

/* Leapfrog of a batch (k_leapfrog per replica, one thread per (atom, axis)):
 * Berendsen scale, box and skin of the block's replica. */
__global__ void __launch_bounds__(3 * MD_LA) k_leapfrog_b(md_kparams kp, thermo_par tp,
                                                         step_io io, int nrep,
                                                         const int2 *__restrict__ tab,
                                                         const md_rep *__restrict__ reps,
                                                         md_repstate *repst, int *rep_upd,
                                                         unsigned long long *racc,
                                                         double *x, double *v,
                                                         const double *__restrict__ mass,
                                                         const double *__restrict__ kick,
                                                         float4 *pos4,
                                                         const long long *__restrict__ f,
                                                         const float *__restrict__ epot,
                                                         const float *__restrict__ vir)
{
    __shared__ double sh[3 * MD_LA / 32];
    __shared__ long long shl[3 * (3 * MD_LA / 32)];
    __shared__ float s_x[3][MD_LA];
    pdl_wait();   /* the forces of this step */
    const int2 bt = tab[blockIdx.x];
    const md_rep &R = reps[bt.x];
    const int d = threadIdx.x / MD_LA, a = threadIdx.x - d * MD_LA;
    const int s = bt.y + a;
    const bool act = s < R.atom0 + R.natom;
    const size_t o = (size_t)d * kp.pitch + s;
    double ke2 = 0.0, pe = 0.0, w = 0.0;
    if (act) {
        axis_par ax = axis_of(d, R.wlim, R.boxd, R.box2i);
        double vv = v[o] + (double)f[o] * kick[s];
        if (tp.berendsen) vv *= repst[bt.x].lam_next;
        v[o] = vv;
        double xx = x[o] + vv * kp.dt;
        if (tp.npt) {
            /* Berendsen barostat: positions and box scaled by the factor the
             * last step's pressure gave; wrap into the scaled box */
            const double mu = repst[bt.x].mu_next;
            xx *= mu;
            ax.L *= mu;
            ax.two_over_l = 2.0 / ax.L;
            ax.lim = 0.4999f * (float)ax.L;
        }
        s_x[d][a] = wrap(xx, ax.lim, ax.L, ax.two_over_l);
        x[o] = xx;
        ke2 = mass[s] * (vv * vv);
        if (d == 0 && tp.energy) pe = epot[s];
        if (d == 0 && (tp.energy || tp.npt)) w = vir[s];
    }
    __syncthreads();
    if (d == 0 && act) {
        float4 p = make_float4(s_x[0][a], s_x[1][a], s_x[2][a], pos4[s].w);
        pos4[s] = p;
        if (md_rsq_box(p, io.pos_old[s], R.box, R.boxi) >= R.rmaxdif) {
            io.st->update = 1;
            rep_upd[bt.x] = 1;
        }
    }
    block_fix_add(ke2, pe, w, tp.energy || tp.npt, racc + 3 * bt.x, shl);
    if (md_last_block(io.counter)) {
        finalize_b(kp, tp, 0, nrep, reps, repst, racc, io.st, io.rec, io.rec_cap, io.rep_hist, sh);
        if (threadIdx.x == 0) {
            set_condition(io);
            *io.counter = 0;
        }
    }
}

/* Velocity Verlet first half of a batch (k_vv_first per replica). */
__global__ void __launch_bounds__(3 * MD_LA) k_vv_first_b(md_kparams kp, step_io io,
                                                         const int2 *__restrict__ tab,
                                                         const md_rep *__restrict__ reps,
                                                         const md_repstate *__restrict__ repst,
                                                         int *rep_upd, double *x, double *v,
                                                         const double *__restrict__ kick,
                                                         float4 *pos4,
                                                         const long long *__restrict__ f)
{
    __shared__ float s_x[3][MD_LA];
    const int2 bt = tab[blockIdx.x];
    const md_rep &R = reps[bt.x];
    const int d = threadIdx.x / MD_LA, a = threadIdx.x - d * MD_LA;
    const int s = bt.y + a;
    const bool act = s < R.atom0 + R.natom;
    const size_t o = (size_t)d * kp.pitch + s;
    const double scale = repst[bt.x].kick_scale;
    if (act) {
        const axis_par ax = axis_of(d, R.wlim, R.boxd, R.box2i);
        double vv = v[o];
        if (scale != 1.0) vv *= scale;
        vv += (double)f[o] * (0.5 * kick[s]);
        v[o] = vv;
        double xx = x[o] + vv * kp.dt;
        s_x[d][a] = wrap(xx, ax.lim, ax.L, ax.two_over_l);
        x[o] = xx;
    }
    __syncthreads();
    if (d == 0 && act) {
        float4 p = make_float4(s_x[0][a], s_x[1][a], s_x[2][a], pos4[s].w);
        pos4[s] = p;
        if (md_rsq_box(p, io.pos_old[s], R.box, R.boxi) >= R.rmaxdif) {
            io.st->update = 1;
            rep_upd[bt.x] = 1;
        }
    }
    if (md_last_block(io.counter)) {
        if (threadIdx.x == 0) {
            set_condition(io);
            *io.counter = 0;
        }
    }
}

/* Velocity Verlet second half of a batch (k_vv_second per replica); do_kick
 * = 0 observes the state only. */
__global__ void __launch_bounds__(3 * MD_LA) k_vv_second_b(md_kparams kp, thermo_par tp,
                                                          int do_kick, step_io io, int nrep,
                                                          const int2 *__restrict__ tab,
                                                          const md_rep *__restrict__ reps,
                                                          md_repstate *repst,
                                                          unsigned long long *racc, double *v,
                                                          const double *__restrict__ mass,
                                                          const double *__restrict__ kick,
                                                          const long long *__restrict__ f,
                                                          const float *__restrict__ epot,
                                                          const float *__restrict__ vir)
{
    __shared__ double sh[3 * MD_LA / 32];
    __shared__ long long shl[3 * (3 * MD_LA / 32)];
    pdl_wait();   /* the forces of this step */
    const int2 bt = tab[blockIdx.x];
    const md_rep &R = reps[bt.x];
    const int d = threadIdx.x / MD_LA, a = threadIdx.x - d * MD_LA;
    const int s = bt.y + a;
    const size_t o = (size_t)d * kp.pitch + s;
    double ke2 = 0.0, pe = 0.0, w = 0.0;
    if (s < R.atom0 + R.natom) {
        double vv = v[o];
        if (do_kick) {
            vv += (double)f[o] * (0.5 * kick[s]);
            v[o] = vv;
        } else {
            vv *= repst[bt.x].vscale;
        }
        ke2 = mass[s] * (vv * vv);
        if (d == 0 && tp.energy) { pe = epot[s]; w = vir[s]; }
    }
    block_fix_add(ke2, pe, w, tp.energy, racc + 3 * bt.x, shl);
    if (md_last_block(io.counter)) {
        finalize_b(kp, tp, do_kick ? 1 : 2, nrep, reps, repst, racc, io.st, io.rec, io.rec_cap, io.rep_hist, sh);
        if (threadIdx.x == 0) *io.counter = 0;
    }
}

/* NPT: after a leapfrog step, one thread per replica scales the replica's box
 * by the factor the step applied to its positions (mu_used) and refreshes
 * what the kernels derive from it: the FP32 box and its inverse as the
 * reference rounds it (simulation.cu:290-292), 2/L, the wrap limit and the
 * cell side.  The cell grid keeps its cell counts and stencil until the
 * host lays it out again (md_step does between chunks of at most 128
 * steps, before the grid's 3% margin can be used up at the per-step clamp
 * of mu, 1e-4), so a box whose cells shrink below half the list radius
 * inside a chunk, or whose list radius exceeds half the box, can no longer
 * be listed correctly: that sets the sticky status 2, which the host
 * reports. */
__global__ void k_npt_box_b(int nrep, md_rep *reps, const md_repstate *__restrict__ repst, md_devstate *st)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrep) return;
    md_rep &R = reps[r];
    if (!R.npt) return;
    const double mu = repst[r].mu_used;
    bool bad = false;
    for (int d = 0; d < 3; d++) {
        const double L = R.boxd[d] * mu;
        R.boxd[d] = L;
        R.box[d] = (float)L;
        R.boxi[d] = (float)(1.0 / L);
        R.box2i[d] = 2.0 / L;
        R.wlim[d] = 0.4999f * R.box[d];
        R.binlen[d] = R.box[d] / (float)R.ncell[d];
        if (R.stencil[d] >= 0 && R.binlen[d] < R.rl_half) bad = true;
        if (2.0f * R.rl_half > 0.5f * R.box[d]) bad = true;
    }
    if (bad) atomicOr(&st->status, 2);
}

template <int KIND, bool ENERGY>
void pair_dispatch_b(md_ctx *c, const md_kparams &kp)
{
    const int k = md_grid_index(128 / c->pair_tpa);
    const int2 *tab = c->grid_tab + c->grid_off[k];
    const int nb = c->grid_cnt[k];
    switch (c->pair_tpa * 100 + md_pair_depth(c)) {
#define MD_PAIR_B_CASE(T, BB)                                                                    \
    case T * 100 + BB:                                                                           \
        k_pair_b<KIND, T, BB, ENERGY><<<nb, 128, 0, c->stream>>>(                                \
            kp.cap, kp.pitch, kp.centered, tab, c->reps_dev, c->ljr_dev, c->pos4, c->type, c->nl, \
            c->nl_n, c->f, c->vir, c->epot);                                                     \
        break;
        MD_PAIR_B_CASE(1, 8)
        MD_PAIR_B_CASE(2, 8)
        MD_PAIR_B_CASE(4, 4)
        MD_PAIR_B_CASE(4, 8)
        MD_PAIR_B_CASE(8, 2)
        MD_PAIR_B_CASE(8, 4)
        MD_PAIR_B_CASE(16, 1)
        MD_PAIR_B_CASE(16, 2)
        MD_PAIR_B_CASE(32, 1)
#undef MD_PAIR_B_CASE
    default:
        break;
    }
}

inline const int2 *grid_int(const md_ctx *c) { return c->grid_tab + c->grid_off[md_grid_index(MD_LA)]; }
inline int grid_int_blocks(const md_ctx *c) { return c->grid_cnt[md_grid_index(MD_LA)]; }

}  // namespace

void launch_forces_b(md_ctx *c, const md_kparams &kp, bool energy, int terms)
{
    if ((terms & MD_TERM_PAIR) && c->fp64) {
        launch_pair64(c, energy);
    } else if (terms & MD_TERM_PAIR) {
        if (c->lkspace == 0) {
            if (energy) pair_dispatch_b<0, true>(c, kp);
            else pair_dispatch_b<0, false>(c, kp);
        } else {
            if (energy) pair_dispatch_b<1, true>(c, kp);
            else pair_dispatch_b<1, false>(c, kp);
        }
    } else {
        cudaMemsetAsync(c->f, 0, sizeof(long long) * 3 * (size_t)c->pitch, c->stream);
        cudaMemsetAsync(c->vir, 0, sizeof(float) * (size_t)c->pitch, c->stream);
        cudaMemsetAsync(c->epot, 0, sizeof(float) * (size_t)c->pitch, c->stream);
    }
    launch_bonded(c, kp, energy, terms);
}

void launch_leapfrog_b(md_ctx *c, const md_kparams &kp, int energy, unsigned long long cond,
                       int has_cond)
{
    struct npt_after {   /* the box follows the positions the step scaled */
        md_ctx *c;
        ~npt_after()
        {
            if (c->enstype == 2) launch_npt_box_b(c);
        }
    } after{c};
    md_launch_pdl(k_leapfrog_b, dim3(grid_int_blocks(c)), dim3(3 * MD_LA), c->stream, kp,
                  make_tp(c, energy), make_io(c, cond, has_cond), c->nrep, grid_int(c),
                  (const md_rep *)c->reps_dev, c->repst, c->rep_upd, c->racc, c->x, c->v,
                  (const double *)c->mass, (const double *)c->kick, c->pos4,
                  (const long long *)c->f, (const float *)c->epot, (const float *)c->vir);
}

void launch_npt_box_b(md_ctx *c)
{
    k_npt_box_b<<<(c->nrep + 127) / 128, 128, 0, c->stream>>>(c->nrep, c->reps_dev, c->repst, c->st);
}

void launch_vv_first_b(md_ctx *c, const md_kparams &kp, unsigned long long cond, int has_cond)
{
    k_vv_first_b<<<grid_int_blocks(c), 3 * MD_LA, 0, c->stream>>>(kp, make_io(c, cond, has_cond),
                                                           grid_int(c), c->reps_dev, c->repst,
                                                           c->rep_upd, c->x, c->v, c->kick, c->pos4,
                                                           c->f);
}

void launch_vv_second_b(md_ctx *c, const md_kparams &kp, int energy, int kick)
{
    md_launch_pdl(k_vv_second_b, dim3(grid_int_blocks(c)), dim3(3 * MD_LA), c->stream, kp,
                  make_tp(c, energy), kick, make_io(c, 0, 0), c->nrep, grid_int(c),
                  (const md_rep *)c->reps_dev, c->repst, c->racc, c->v, (const double *)c->mass,
                  (const double *)c->kick, (const long long *)c->f, (const float *)c->epot,
                  (const float *)c->vir);
}
