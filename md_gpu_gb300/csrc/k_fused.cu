/*
 * k_fused.cu -- one kernel per leapfrog step for systems without bonded
 * terms: pair forces (pair_forces.cu:133-205 / :34-131), then in the same
 * thread the leapfrog update of that atom (nve_leapfrog.cu:31-60,
 * nvt_leapfrog_ber.cu:29-80), the next step's list check
 * (neighborlist.cu:157-176) and the FP64 kinetic-energy partial; the last
 * block to finish turns the step's sums into T and sets the rebuild condition.
 *
 * Positions are double buffered: the step reads pos4 and writes the updated
 * copy to pos4_next, so no thread sees a neighbour that has already moved.
 * The forces never leave the registers except for the copy kept for
 * read-out.
 */
#include "md_pair.cuh"
#include "md_thermo.cuh"

namespace {

template <int KIND, int TPA, int B>
__global__ void __launch_bounds__(128) k_pair_leapfrog(
    md_kparams kp, pair_consts pc, thermo_par tp, step_io io, const float4 *__restrict__ pos4,
    float4 *__restrict__ pos4_next, const int *__restrict__ type, const unsigned *__restrict__ nl,
    const int *__restrict__ nl_n, const float2 *__restrict__ ljtab, long long *f, float *vir,
    double *x, double *v, const double *__restrict__ mass, const double *__restrict__ kick)
{
    constexpr int NA = 128 / TPA;   /* atoms per block */
    __shared__ float2 lj[MD_MAXTYPE * MD_MAXTYPE];
    __shared__ long long sh[12];   /* 3 integers per warp */
    __shared__ long long s_f[NA][3];
    __shared__ float s_x[NA][3];
    if (threadIdx.x < MD_MAXTYPE * MD_MAXTYPE) lj[threadIdx.x] = ljtab[threadIdx.x];
    __syncthreads();
    int gt = blockIdx.x * blockDim.x + threadIdx.x;
    int i = gt / TPA, lane = gt % TPA;
    bool active = i < kp.n;
    pair_total t = pair_sum<KIND, TPA, B, false>(geom_kp{kp, pc}, kp.cap, active ? i : 0, active, lane, pos4, type,
                                                 nl, nl_n, lj);
    const size_t P = (size_t)kp.pitch;
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
    __syncthreads();
    /* FP64 leapfrog of the block's atoms spread over all threads, one
     * (atom, axis) per thread: full warps on the FP64 pipe */
    const int i0 = blockIdx.x * NA;
    const double lam = tp.berendsen ? io.st->lam_next : 1.0;
    double ke2 = 0.0;
    for (int k = threadIdx.x; k < 3 * NA; k += blockDim.x) {
        int a = k / 3, d = k - 3 * a, ia = i0 + a;
        if (ia < kp.n) {
            double vv = v[d * P + ia] + (double)s_f[a][d] * kick[ia];
            if (tp.berendsen) vv *= lam;
            v[d * P + ia] = vv;
            double xx = x[d * P + ia] + vv * kp.dt;
            s_x[a][d] = wrap(xx, kp.wlim[d], kp.boxd[d], kp.box2i[d]);
            x[d * P + ia] = xx;
            ke2 += mass[ia] * vv * vv;
        }
    }
    __syncthreads();
    if (threadIdx.x < NA) {
        int ia = i0 + threadIdx.x;
        if (ia < kp.n) {
            float4 p = make_float4(s_x[threadIdx.x][0], s_x[threadIdx.x][1], s_x[threadIdx.x][2],
                                   pos4[ia].w);
            pos4_next[ia] = p;
            check_moved(p, io.pos_old[ia], kp, io.st);
        }
    }
    block_fix_add(ke2, 0.0, 0.0, 0, io.st->acc, sh);
    if (md_last_block(io.counter)) {
        finalize(kp, tp, 0, io.st, io.rec, io.rec_cap);
        if (threadIdx.x == 0) {
            set_condition(io);
            *io.counter = 0;
        }
    }
}

template <int KIND>
void fused_dispatch(md_ctx *c, const md_kparams &kp, const pair_consts &pc, const thermo_par &tp,
                    const step_io &io)
{
    long long threads = (long long)kp.n * c->pair_tpa;
    int nb = (int)((threads + 127) / 128);
    const float2 *lj = (const float2 *)c->lj_dev;
    switch (c->pair_tpa) {
#define MD_FUSED_CASE(T)                                                                         \
    case T:                                                                                      \
        k_pair_leapfrog<KIND, T, (T >= 32 ? 1 : (T >= 16 ? 2 : (T >= 8 ? 4 : 8)))>              \
            <<<nb, 128, 0, c->stream>>>(kp, pc, tp, io, c->pos4, c->pos4_alt, c->type, c->nl,    \
                                        c->nl_n, lj, c->f, c->vir, c->x, c->v, c->mass, c->kick); \
        break;
        MD_FUSED_CASE(1)
        MD_FUSED_CASE(2)
        MD_FUSED_CASE(4)
        MD_FUSED_CASE(8)
        MD_FUSED_CASE(16)
        MD_FUSED_CASE(32)
#undef MD_FUSED_CASE
    default:
        break;
    }
}

}  // namespace

bool md_can_fuse(const md_ctx *c)
{
    return c->fuse_step && !c->batch && c->integrator == MD_LEAPFROG && !c->has_bonds &&
           !c->has_angles;
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
