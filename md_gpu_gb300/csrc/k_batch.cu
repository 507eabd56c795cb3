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
 * memory), and the block partials of the FP64 reductions split cleanly by
 * replica.  The arithmetic per atom is the single-system arithmetic
 * (pair_sum, the leapfrog / velocity-Verlet updates of k_integrate.cu), so a
 * replica advances bit-for-bit as it would alone with the same tuning.
 */
#include "md_pair.cuh"
#include "md_thermo.cuh"

namespace {

__device__ __forceinline__ geom_reg rep_geom(const md_rep &R)
{
    geom_reg g;
    for (int d = 0; d < 3; d++) {
        g.L_[d] = R.box[d];
        g.Li_[d] = R.boxi[d];
    }
    g.rcsq_ = R.rcutsq;
    g.reacf_ = R.reacf;
    g.palfa_ = R.palfa;
    g.spiialfa_ = R.spiialfa;
    g.alfasq_ = R.alfasq;
    g.wolf_ = R.wolf;
    g.ucc_ = R.ucc;
    g.rc6i_ = R.rc6i;
    g.rcinv_ = R.rcinv;
    return g;
}

/* Pair forces of a batch: block b holds 128/TPA atoms of replica tab[b].x
 * starting at tab[b].y. */
template <int KIND, int TPA, int B, bool ENERGY>
__global__ void __launch_bounds__(128) k_pair_b(int cap, int pitch, const int2 *__restrict__ tab,
                                                const md_rep *__restrict__ reps,
                                                const float2 *__restrict__ ljr,
                                                const float4 *__restrict__ pos4,
                                                const int *__restrict__ type,
                                                const unsigned *__restrict__ nl,
                                                const int *__restrict__ nl_n, long long *f,
                                                float *vir, float *epot)
{
    __shared__ float2 lj[MD_MAXTYPE * MD_MAXTYPE];
    const int2 bt = tab[blockIdx.x];
    const md_rep &R = reps[bt.x];
    if (threadIdx.x < MD_MAXTYPE * MD_MAXTYPE)
        lj[threadIdx.x] = ljr[bt.x * MD_MAXTYPE * MD_MAXTYPE + threadIdx.x];
    const geom_reg g = rep_geom(R);
    const int end = R.atom0 + R.natom;
    __syncthreads();
    const int i = bt.y + (int)threadIdx.x / TPA, lane = (int)threadIdx.x % TPA;
    const bool active = i < end;
    pair_total t = pair_sum<KIND, TPA, B, ENERGY>(g, cap, active ? i : bt.y, active, lane, pos4,
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

/* Per-replica FP64 totals from the block partials (each replica's blocks
 * are one contiguous range of the 256-atom grid), one warp per replica in a
 * fixed order, then each replica's thermostat bookkeeping and the batch's
 * step record (sums over replicas).  Runs in the last block to finish. */
__device__ void finalize_b(const md_kparams &kp, const thermo_par &tp, int mode, int nrep,
                           const md_rep *__restrict__ reps, md_repstate *repst,
                           const double *partials, int npart, md_devstate *st, md_thermo *rec,
                           int rec_cap, double *sh)
{
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    double tke = 0.0, tpe = 0.0, tw = 0.0, tex = 0.0;
    for (int r = w; r < nrep; r += nw) {
        const md_rep &R = reps[r];
        double a = 0.0, b = 0.0, c = 0.0;
        for (int k = lane; k < R.nblk; k += 32) {
            a += __ldcg(partials + R.blk0 + k);
            if (tp.energy) {
                b += __ldcg(partials + npart + R.blk0 + k);
                c += __ldcg(partials + 2 * npart + R.blk0 + k);
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
            c += __shfl_down_sync(0xffffffffu, c, o);
        }
        if (lane == 0) {
            thermo_par t = tp;
            t.t0 = R.t0;
            t.ndf = R.ndf;
            t.q_nh = R.q_nh;
            double xi, eta, lam;
            double ke = thermo_advance(kp.dt, t, mode, a, b, c, repst + r, &xi, &eta, &lam);
            tke += ke;
            tpe += b;
            tw += c;
            if (t.nh) tex += 0.5 * t.q_nh * xi * xi + t.ndf * RGAS * t.t0 * eta;
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
    st->temper = 2.0 * KE / (tp.ndf * RGAS);
    write_record(tp, tp.ndf, KE, PE, W, EX, 0.0, 1.0, st, rec, rec_cap);
}

/* Leapfrog of a batch (k_leapfrog per replica): Berendsen scale, box and
 * skin of the block's replica. */
__global__ void __launch_bounds__(256) k_leapfrog_b(md_kparams kp, thermo_par tp, step_io io,
                                                    int nrep, const int2 *__restrict__ tab,
                                                    const md_rep *__restrict__ reps,
                                                    md_repstate *repst, int *rep_upd, double *x,
                                                    double *v, const double *__restrict__ mass,
                                                    const double *__restrict__ minv, float4 *pos4,
                                                    const long long *__restrict__ f,
                                                    const float *__restrict__ epot,
                                                    const float *__restrict__ vir)
{
    __shared__ double sh[8];
    const int2 bt = tab[blockIdx.x];
    const md_rep &R = reps[bt.x];
    const int s = bt.y + threadIdx.x;
    const int P = kp.pitch;
    const double lam = tp.berendsen ? repst[bt.x].lam_next : 1.0;
    double ke = 0.0, pe = 0.0, w = 0.0;
    if (s < R.atom0 + R.natom) {
        double m = mass[s], dtm = kp.dt * minv[s];
        double xn[3];
        for (int d = 0; d < 3; d++) {
            double F = (double)f[d * P + s] * FX_INV;
            double vv = (v[d * P + s] + F * dtm) * lam;
            v[d * P + s] = vv;
            double xx = wrap(x[d * P + s] + vv * kp.dt, R.boxd[d], R.box2i[d]);
            x[d * P + s] = xx;
            xn[d] = xx;
            ke += vv * vv;
        }
        ke *= 0.5 * m;
        float4 p = pos4[s];
        p = make_float4((float)xn[0], (float)xn[1], (float)xn[2], p.w);
        pos4[s] = p;
        if (md_rsq_box(p, io.pos_old[s], R.box, R.boxi) >= R.rmaxdif) {
            io.st->update = 1;
            rep_upd[bt.x] = 1;
        }
        if (tp.energy) { pe = epot[s]; w = vir[s]; }
    }
    write_partials(ke, pe, w, tp.energy, io.partials, sh);
    if (md_last_block(io.counter)) {
        finalize_b(kp, tp, 0, nrep, reps, repst, io.partials, gridDim.x, io.st, io.rec, io.rec_cap, sh);
        if (threadIdx.x == 0) {
            set_condition(io);
            *io.counter = 0;
        }
    }
}

/* Velocity Verlet first half of a batch (k_vv_first per replica). */
__global__ void __launch_bounds__(256) k_vv_first_b(md_kparams kp, step_io io,
                                                    const int2 *__restrict__ tab,
                                                    const md_rep *__restrict__ reps,
                                                    const md_repstate *__restrict__ repst,
                                                    int *rep_upd, double *x, double *v,
                                                    const double *__restrict__ minv, float4 *pos4,
                                                    const long long *__restrict__ f)
{
    const int2 bt = tab[blockIdx.x];
    const md_rep &R = reps[bt.x];
    const int s = bt.y + threadIdx.x;
    const int P = kp.pitch;
    const double scale = repst[bt.x].kick_scale;
    if (s < R.atom0 + R.natom) {
        double hdtm = 0.5 * kp.dt * minv[s];
        double xn[3];
        for (int d = 0; d < 3; d++) {
            double F = (double)f[d * P + s] * FX_INV;
            double vv = v[d * P + s] * scale + F * hdtm;
            v[d * P + s] = vv;
            double xx = wrap(x[d * P + s] + vv * kp.dt, R.boxd[d], R.box2i[d]);
            x[d * P + s] = xx;
            xn[d] = xx;
        }
        float4 p = pos4[s];
        p = make_float4((float)xn[0], (float)xn[1], (float)xn[2], p.w);
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

/* Velocity Verlet second half of a batch (k_vv_second per replica); kick = 0
 * observes the state only. */
__global__ void __launch_bounds__(256) k_vv_second_b(md_kparams kp, thermo_par tp, int kick,
                                                     step_io io, int nrep,
                                                     const int2 *__restrict__ tab,
                                                     const md_rep *__restrict__ reps,
                                                     md_repstate *repst, double *v,
                                                     const double *__restrict__ mass,
                                                     const double *__restrict__ minv,
                                                     const long long *__restrict__ f,
                                                     const float *__restrict__ epot,
                                                     const float *__restrict__ vir)
{
    __shared__ double sh[8];
    const int2 bt = tab[blockIdx.x];
    const md_rep &R = reps[bt.x];
    const int s = bt.y + threadIdx.x;
    const int P = kp.pitch;
    double ke = 0.0, pe = 0.0, w = 0.0;
    const double scale = kick ? 1.0 : repst[bt.x].vscale;
    if (s < R.atom0 + R.natom) {
        double m = mass[s], hdtm = 0.5 * kp.dt * minv[s];
        for (int d = 0; d < 3; d++) {
            double vv = v[d * P + s];
            if (kick) {
                vv += (double)f[d * P + s] * FX_INV * hdtm;
                v[d * P + s] = vv;
            } else {
                vv *= scale;
            }
            ke += vv * vv;
        }
        ke *= 0.5 * m;
        if (tp.energy) { pe = epot[s]; w = vir[s]; }
    }
    write_partials(ke, pe, w, tp.energy, io.partials, sh);
    if (md_last_block(io.counter)) {
        finalize_b(kp, tp, kick ? 1 : 2, nrep, reps, repst, io.partials, gridDim.x, io.st, io.rec,
                   io.rec_cap, sh);
        if (threadIdx.x == 0) *io.counter = 0;
    }
}

template <int KIND, bool ENERGY>
void pair_dispatch_b(md_ctx *c, const md_kparams &kp)
{
    const int k = md_grid_index(128 / c->pair_tpa);
    const int2 *tab = c->grid_tab + c->grid_off[k];
    const int nb = c->grid_cnt[k];
    switch (c->pair_tpa) {
#define MD_PAIR_B_CASE(T)                                                                        \
    case T:                                                                                      \
        k_pair_b<KIND, T, (T >= 32 ? 1 : (T >= 16 ? 2 : (T >= 8 ? 4 : 8))), ENERGY>             \
            <<<nb, 128, 0, c->stream>>>(kp.cap, kp.pitch, tab, c->reps_dev, c->ljr_dev, c->pos4, \
                                        c->type, c->nl, c->nl_n, c->f, c->vir, c->epot);         \
        break;
        MD_PAIR_B_CASE(1)
        MD_PAIR_B_CASE(2)
        MD_PAIR_B_CASE(4)
        MD_PAIR_B_CASE(8)
        MD_PAIR_B_CASE(16)
        MD_PAIR_B_CASE(32)
#undef MD_PAIR_B_CASE
    default:
        break;
    }
}

inline const int2 *grid256(const md_ctx *c) { return c->grid_tab + c->grid_off[md_grid_index(256)]; }
inline int grid256_blocks(const md_ctx *c) { return c->grid_cnt[md_grid_index(256)]; }

}  // namespace

void launch_forces_b(md_ctx *c, const md_kparams &kp, bool energy, int terms)
{
    if (terms & MD_TERM_PAIR) {
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
}

void launch_leapfrog_b(md_ctx *c, const md_kparams &kp, int energy, unsigned long long cond,
                       int has_cond)
{
    k_leapfrog_b<<<grid256_blocks(c), 256, 0, c->stream>>>(
        kp, make_tp(c, energy), make_io(c, cond, has_cond), c->nrep, grid256(c), c->reps_dev,
        c->repst, c->rep_upd, c->x, c->v, c->mass, c->minv, c->pos4, c->f, c->epot, c->vir);
}

void launch_vv_first_b(md_ctx *c, const md_kparams &kp, unsigned long long cond, int has_cond)
{
    k_vv_first_b<<<grid256_blocks(c), 256, 0, c->stream>>>(kp, make_io(c, cond, has_cond),
                                                           grid256(c), c->reps_dev, c->repst,
                                                           c->rep_upd, c->x, c->v, c->minv, c->pos4,
                                                           c->f);
}

void launch_vv_second_b(md_ctx *c, const md_kparams &kp, int energy, int kick)
{
    k_vv_second_b<<<grid256_blocks(c), 256, 0, c->stream>>>(
        kp, make_tp(c, energy), kick, make_io(c, 0, 0), c->nrep, grid256(c), c->reps_dev,
        c->repst, c->v, c->mass, c->minv, c->f, c->epot, c->vir);
}
