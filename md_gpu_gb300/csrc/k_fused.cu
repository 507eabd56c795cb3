/*
 * k_fused.cu -- one kernel per leapfrog step for systems without bonded
 * terms: pair forces (pair_forces.cu:133-205 / :34-131), then in the same
 * thread the leapfrog update of that atom (nve_leapfrog.cu:31-60,
 * nvt_leapfrog_ber.cu:29-80), the next step's list check
 * (neighborlist.cu:157-176) and the kinetic-energy sums; the last block to
 * finish turns the step's sums into T and sets the rebuild condition.  The
 * update's inputs (x, v, 1/m, m, the positions at the last build) are copied
 * into shared memory with cp.async at the start, so they arrive while the
 * block computes its pair forces.
 *
 * Positions are double buffered: the step reads pos4 and writes the updated
 * copy to pos4_next, so no thread sees a neighbour that has already moved.
 * The forces never leave the registers except for the copy kept for
 * read-out.
 */
#include "md_pair.cuh"
#include "md_thermo.cuh"

namespace {

constexpr int FUSED_THREADS = 128;   /* threads per block */

template <int KIND, int TPA, int B>
__global__ void __launch_bounds__(FUSED_THREADS) k_pair_leapfrog(
    md_kparams kp, pair_consts pc, thermo_par tp, step_io io, const float4 *__restrict__ pos4,
    float4 *__restrict__ pos4_next, const int *__restrict__ type, const unsigned *__restrict__ nl,
    const int *__restrict__ nl_n, const float2 *__restrict__ ljtab, long long *f, float *vir,
    double *x, double *v, const double *__restrict__ mass, const double *__restrict__ kick)
{
    constexpr int NA = FUSED_THREADS / TPA;   /* atoms per block */
    __shared__ float2 lj[MD_MAXTYPE * MD_MAXTYPE];
    __shared__ long long sh[3 * FUSED_THREADS / 32];   /* 3 integers per warp */
    __shared__ long long s_f[NA][3];
    __shared__ double s_x0[3][NA], s_v0[3][NA], s_kick[NA], s_mass[NA];
    __shared__ float4 s_old[NA];
    __shared__ float s_x[NA][3];
    pdl_trigger();   /* the list passes that follow may be scheduled */
    const int i0 = blockIdx.x * NA;
    const size_t P = (size_t)kp.pitch;
    /* the update's inputs travel while the pair forces are computed */
    for (int k = threadIdx.x; k < 3 * NA; k += blockDim.x) {
        const int d = k / NA, a = k - d * NA, ia = i0 + a;
        if (ia < kp.n) {
            cp_async8(&s_x0[d][a], x + d * P + ia);
            cp_async8(&s_v0[d][a], v + d * P + ia);
        }
    }
    if (threadIdx.x < NA && i0 + (int)threadIdx.x < kp.n) {
        const int ia = i0 + threadIdx.x;
        cp_async8(&s_kick[threadIdx.x], kick + ia);
        cp_async8(&s_mass[threadIdx.x], mass + ia);
        cp_async16(&s_old[threadIdx.x], io.pos_old + ia);
    }
    if (threadIdx.x < MD_MAXTYPE * MD_MAXTYPE) lj[threadIdx.x] = ljtab[threadIdx.x];
    __syncthreads();
    int gt = blockIdx.x * blockDim.x + threadIdx.x;
    int i = gt / TPA, lane = gt % TPA;
    bool active = i < kp.n;
    /* the pair loop of k_pair (entries two at a time in packed f32x2
     * instructions for even B), so both step forms sum the same forces bit
     * for bit: 76.3 against 78.7 us per step on 64000 ions with the scalar
     * loop */
    pair_total t = pair_sum<KIND, TPA, B, false, true>(geom_kp{kp, pc}, kp.cap, active ? i : 0, active, lane, pos4, type,
                                                 nl, nl_n, lj);
    if (lane == 0) {
        int a = threadIdx.x / TPA;
        s_f[a][0] = t.fx;
        s_f[a][1] = t.fy;
        s_f[a][2] = t.fz;
        if (active) {
            f[i] = t.fx;
            f[P + i] = t.fy;
            f[2 * P + i] = t.fz;
            vir[i] = t.fw;
        }
    }
    cp_async_wait();
    __syncthreads();
    /* FP64 leapfrog of the block's atoms, one (atom, axis) per thread, the
     * same operations as k_leapfrog */
    const double lam = tp.berendsen ? io.st->lam_next : 1.0;
    long long ke = 0;
    for (int k = threadIdx.x; k < 3 * NA; k += blockDim.x) {
        const int d = k / NA, a = k - d * NA, ia = i0 + a;
        if (ia < kp.n) {
            const axis_par ax = axis_of(d, kp.wlim, kp.boxd, kp.box2i);
            double vv = s_v0[d][a] + (double)s_f[a][d] * s_kick[a];
            if (tp.berendsen) vv *= lam;
            v[d * P + ia] = vv;
            double xx = s_x0[d][a] + vv * kp.dt;
            s_x[a][d] = wrap(xx, ax.lim, ax.L, ax.two_over_l);
            x[d * P + ia] = xx;
            ke += ke_fix(s_mass[a], vv);
        }
    }
    __syncthreads();
    bool moved = false;
    if (threadIdx.x < NA) {
        int ia = i0 + threadIdx.x;
        if (ia < kp.n) {
            float4 p = make_float4(s_x[threadIdx.x][0], s_x[threadIdx.x][1], s_x[threadIdx.x][2],
                                   pos4[ia].w);
            pos4_next[ia] = p;
            moved = md_rsq_exact(p, s_old[threadIdx.x], kp) >= kp.rmaxdif;
        }
    }
    if (block_close(ke, 0, 0, 1, moved, io.st, io.counter, sh)) {
        finalize(kp, tp, 0, io.st, io.rec, io.rec_cap);
        set_condition(io);
        *io.counter = 0;
    }
}

template <int KIND>
void fused_dispatch(md_ctx *c, const md_kparams &kp, const pair_consts &pc, const thermo_par &tp,
                    const step_io &io)
{
    long long threads = (long long)kp.n * c->pair_tpa;
    int nb = (int)((threads + FUSED_THREADS - 1) / FUSED_THREADS);
    const float2 *lj = (const float2 *)c->lj_dev;
    switch (c->pair_tpa * 100 + md_pair_depth(c)) {
#define MD_FUSED_CASE(T, BB)                                                                     \
    case T * 100 + BB:                                                                           \
        k_pair_leapfrog<KIND, T, BB><<<nb, FUSED_THREADS, 0, c->stream>>>(                                 \
            kp, pc, tp, io, c->pos4, c->pos4_alt, c->type, c->nl, c->nl_n, lj, c->f, c->vir,     \
            c->x, c->v, c->mass, c->kick);                                                       \
        break;
        MD_FUSED_CASE(1, 8)
        MD_FUSED_CASE(2, 8)
        MD_FUSED_CASE(4, 4)
        MD_FUSED_CASE(4, 8)
        MD_FUSED_CASE(8, 2)
        MD_FUSED_CASE(8, 4)
        MD_FUSED_CASE(16, 1)
        MD_FUSED_CASE(16, 2)
        MD_FUSED_CASE(32, 1)
#undef MD_FUSED_CASE
    default:
        break;
    }
}

}  // namespace

bool md_can_fuse(const md_ctx *c)
{
    return c->fuse_step && !c->batch && !c->fp64 && c->integrator == MD_LEAPFROG && !c->has_bonds &&
           !c->has_angles && !c->pme.on;
}

void launch_pair_leapfrog(md_ctx *c, const md_kparams &kp, unsigned long long cond, int has_cond)
{
    pair_consts pc = make_pair_consts(c);
    thermo_par tp = make_tp(c, 0);
    step_io io = make_io(c, cond, has_cond);
    if (c->lkspace == 0) fused_dispatch<0>(c, kp, pc, tp, io);
    else fused_dispatch<1>(c, kp, pc, tp, io);
    /* the updated positions are now the current ones */
    float4 *t = c->pos4;
    c->pos4 = c->pos4_alt;
    c->pos4_alt = t;
}
