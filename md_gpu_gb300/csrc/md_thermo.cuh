/*
 * md_thermo.cuh -- FP64 reductions, step bookkeeping and the list check
 * shared by the integrator kernels.
 */
#ifndef MD_THERMO_CUH
#define MD_THERMO_CUH

#include "md_device.cuh"

namespace {

constexpr double RGAS = 8.314e-3;   /* kJ/mol/K, as integrator.cu:155 (1000/8.314) */

struct thermo_par {
    double t0, tau, q_nh;
    double inv_ndfr;   /* 1 / (ndf R): temperature from 2 KE */
    double inv_q;      /* 1 / Q (Nose-Hoover mass) */
    double dt_tau;     /* dt / tau (Berendsen) */
    int ndf, berendsen, nh, energy;
    int npt;   /* Berendsen barostat (batches): virial summed every step, box scaled */
};

/* Per-step bookkeeping buffers and the graph condition to set. */
struct step_io {
    md_devstate *st;
    md_thermo *rec;
    double *rep_hist;   /* batches: per step and replica (KE, PE, conserved), rec_cap steps */
    int rec_cap;
    unsigned *counter;
    const float4 *pos_old;
    cudaGraphConditionalHandle cond;
    int has_cond;
};

/* Sum of a double over the block; result valid in thread 0. */
__device__ __forceinline__ double block_sum(double v, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) r += sh[k];
    __syncthreads();
    return r;
}

/* x -= L trunc(2x/L) (nve_leapfrog.cu:52-56) with 2/L precomputed; returns
 * the FP32 copy of the result.  An atom whose FP32 position lies inside
 * +-0.4999 L is inside +-L/2 in FP64 as well, where trunc gives 0: only atoms
 * near or past the boundary pay for the FP64 product and trunc (the FP64
 * pipe is the scarce one here), and the result is the same in every case. */
__device__ __forceinline__ float wrap(double &x, float lim, double L, double two_over_l)
{
    float xf = (float)x;
    if (!(fabsf(xf) < lim)) {
        x = x - L * trunc(x * two_over_l);
        xf = (float)x;
    }
    return xf;
}

/* First thermostat half step of the next VV step (NH): from KE (already
 * scaled by the pending factor) and xi, eta; returns the factor s1. */
__device__ __forceinline__ double nh_half_a(double dt, const thermo_par &tp, double ke,
                                            double &xi, double &eta)
{
    double kt = RGAS * tp.t0;
    xi += 0.25 * dt * (2.0 * ke - tp.ndf * kt) * tp.inv_q;
    double s1 = exp(-0.5 * dt * xi);
    ke *= s1 * s1;
    eta += 0.5 * dt * xi;
    xi += 0.25 * dt * (2.0 * ke - tp.ndf * kt) * tp.inv_q;
    return s1;
}

/* The reductions of a step: each thread's twice-kinetic energy ke2 (m v^2,
 * FP64), potential energy and sum ff r^2 are converted once to fixed point
 * (MD_KFIX = 2^32 per kJ/mol for KE, halved in the same conversion; MD_EFIX
 * = 2^24 for the others) and summed
 * with integer shuffles, shared memory and one atomic add per block and
 * quantity.  Integer addition is exact and associative, so the totals do
 * not depend on the order in which threads or blocks contribute, and the
 * slow FP64 pipe only performs one conversion per thread.  sh holds 3
 * integers per warp. */
__device__ __forceinline__ void block_fix_add(double ke2, double pe, double w, int energy,
                                              unsigned long long *acc, long long *sh)
{
    long long a = llrint(ke2 * (0.5 * MD_KFIX));
    long long b = energy ? llrint(pe * MD_EFIX) : 0ll;
    long long c = energy ? llrint(w * MD_EFIX) : 0ll;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        if (energy) {
            b += __shfl_down_sync(0xffffffffu, b, o);
            c += __shfl_down_sync(0xffffffffu, c, o);
        }
    }
    const int wp = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (l == 0) {
        sh[wp] = a;
        sh[nw + wp] = b;
        sh[2 * nw + wp] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long ta = 0, tb = 0, tc = 0;
        for (int k = 0; k < nw; k++) {
            ta += sh[k];
            tb += sh[nw + k];
            tc += sh[2 * nw + k];
        }
        atomicAdd(acc, (unsigned long long)ta);
        if (energy) {
            atomicAdd(acc + 1, (unsigned long long)tb);
            atomicAdd(acc + 2, (unsigned long long)tc);
        }
    }
}

/* One (atom, axis) kinetic-energy term m v^2 / 2 in 2^-32 kJ/mol fixed
 * point, rounded once (the same value block_fix_add takes from m v^2). */
__device__ __forceinline__ long long ke_fix(double m, double vv)
{
    return llrint(m * (vv * vv) * (0.5 * MD_KFIX));
}

/* The end of an integrator block.  Each thread brings its fixed-point terms
 * a (KE, 2^-32 kJ/mol units), b and c (PE, virial, 2^-24; nsum = 3 adds all
 * three, 1 only a, 0 none) and whether its atom moved >= skin/2; the block
 * sums them with integer shuffles, and thread 0 alone adds them to the
 * device state, raises st->update, fences and counts the block.  Returns
 * true in thread 0 of the last block to finish, which then finalises the
 * step.  The other threads' stores (positions, velocities) are read only by
 * later kernels, so they need no fence and their warps leave at once.
 * sh holds 3 integers per warp. */
__device__ __forceinline__ bool block_close(long long a, long long b, long long c, int nsum,
                                            bool moved, md_devstate *st, unsigned *counter,
                                            long long *sh)
{
    if (nsum > 0) {
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            if (nsum > 1) {
                b += __shfl_down_sync(0xffffffffu, b, o);
                c += __shfl_down_sync(0xffffffffu, c, o);
            }
        }
        const int wp = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
        if (l == 0) {
            sh[wp] = a;
            sh[nw + wp] = b;
            sh[2 * nw + wp] = c;
        }
    }
    const int any = __syncthreads_or(moved ? 1 : 0);
    if (threadIdx.x != 0) return false;
    if (nsum > 0) {
        const int nw = blockDim.x >> 5;
        long long ta = 0, tb = 0, tc = 0;
        for (int k = 0; k < nw; k++) {
            ta += sh[k];
            tb += sh[nw + k];
            tc += sh[2 * nw + k];
        }
        atomicAdd(&st->acc[0], (unsigned long long)ta);
        if (nsum > 1) {
            atomicAdd(&st->acc[1], (unsigned long long)tb);
            atomicAdd(&st->acc[2], (unsigned long long)tc);
        }
    }
    if (any) st->update = 1;
    __threadfence();
    return atomicAdd(counter, 1u) == gridDim.x - 1;
}

/* Reads and clears fixed-point accumulators (in the last block, after every
 * block's atomic adds). */
__device__ __forceinline__ double fix_take(unsigned long long *p, double scale)
{
    volatile unsigned long long *v = p;
    const long long x = (long long)*v;
    *v = 0ull;
    return (double)x / scale;
}

/* Thermostat bookkeeping of one system after a step, from its FP64 totals
 * (ke before any pending thermostat scale, pe, w = sum ff r^2).  S is
 * md_devstate (a single system) or md_repstate (one replica of a batch): both
 * hold the same thermostat fields.  mode 0 leapfrog, 1 VV / NH, 2 observe
 * only (no step; the Berendsen reference temperature kept).  Returns the
 * kinetic energy after the thermostat and sets *xi_out, *eta_out, *lam_out. */
template <class S>
__device__ double thermo_advance(double dt, const thermo_par &tp, int mode, double ke, double pe,
                                 double w, S *st, double *xi_out, double *eta_out, double *lam_out)
{
    volatile S *vs = st;
    double kt = RGAS * tp.t0;
    double lam = (mode == 0 && tp.berendsen) ? vs->lam_next : 1.0;
    double xi = vs->xi, eta = vs->eta;
    if (mode == 1) {
        st->vscale = 1.0;
        if (tp.nh) {
            xi = vs->xi_a;
            eta = vs->eta_a;
            xi += 0.25 * dt * (2.0 * ke - tp.ndf * kt) * tp.inv_q;
            double s2 = exp(-0.5 * dt * xi);
            ke *= s2 * s2;
            eta += 0.5 * dt * xi;
            xi += 0.25 * dt * (2.0 * ke - tp.ndf * kt) * tp.inv_q;
            st->vscale = s2;
            st->xi = xi;
            st->eta = eta;
        }
    }
    st->ke = ke;
    if (tp.energy) { st->pe = pe; st->virial = w / 6.0; }
    if (tp.nh && mode != 0) {
        /* the next step's first thermostat half step, from this state */
        double xa = xi, ea = eta;
        double s1 = nh_half_a(dt, tp, ke, xa, ea);
        st->xi_a = xa;
        st->eta_a = ea;
        st->kick_scale = vs->vscale * s1;
    } else if (mode != 0) {
        st->kick_scale = vs->vscale;
    }
    *xi_out = xi;
    *eta_out = eta;
    *lam_out = lam;
    /* observing the state does not move the Berendsen reference temperature:
     * the first step uses T = T0 (integrator.cu:77) */
    if (mode == 2) return ke;
    double temper = 2.0 * ke * tp.inv_ndfr;
    st->temper = temper;
    st->lambda = lam;
    /* integrator.cu:146-147 for the next step, from this step's temperature */
    st->lam_next = tp.berendsen ? sqrt(1.0 + tp.dt_tau * (tp.t0 / temper - 1.0)) : 1.0;
    return ke;
}

/* Appends the record of step `step` (read by the caller before its sums,
 * so the load is not on the path after them) and advances the step counter
 * (thread 0).  rec_cap is a power of two. */
__device__ void write_record(const thermo_par &tp, double inv_ndfr, double ke, double pe, double w,
                             double extra, double xi, double lam, long long step, int builds,
                             md_devstate *st, md_thermo *rec, int rec_cap)
{
    md_thermo r;
    r.step = step;
    r.ke = ke;
    r.temper = 2.0 * ke * inv_ndfr;
    r.pe = tp.energy ? pe : 0.0;
    r.virial = tp.energy ? w / 6.0 : 0.0;
    r.conserved = tp.energy ? ke + pe + extra : 0.0;
    r.xi = xi;
    r.lambda = lam;
    r.builds = builds;
    r.flags = tp.energy ? 1 : 0;
    rec[step & (rec_cap - 1)] = r;
    st->step = step + 1;
}

/* Thread 0 of the last block: the step's totals from the accumulators,
 * temperature, thermostat bookkeeping and the step record (mode as
 * thermo_advance). */
__device__ void finalize(const md_kparams &kp, const thermo_par &tp, int mode, md_devstate *st,
                         md_thermo *rec, int rec_cap)
{
    if (threadIdx.x != 0) return;
    volatile md_devstate *vs = st;
    const long long step = vs->step;
    const int builds = vs->builds;
    double ke = fix_take(&st->acc[0], MD_KFIX);
    double pe = fix_take(&st->acc[1], MD_EFIX);
    double w = fix_take(&st->acc[2], MD_EFIX);
    if (!tp.energy) pe = w = 0.0;
    double xi, eta, lam;
    ke = thermo_advance(kp.dt, tp, mode, ke, pe, w, st, &xi, &eta, &lam);
    if (mode == 2) return;
    double extra = tp.nh ? 0.5 * tp.q_nh * xi * xi + tp.ndf * RGAS * tp.t0 * eta : 0.0;
    write_record(tp, tp.inv_ndfr, ke, pe, w, extra, xi, lam, step, builds, st, rec, rec_cap);
}

/* Per-axis constants of an integrator thread (the axis is a runtime value:
 * selects instead of indexing the parameter arrays). */
struct axis_par {
    double L, two_over_l;
    float lim;
};
__device__ __forceinline__ axis_par axis_of(int d, const float *wlim, const double *boxd,
                                            const double *box2i)
{
    axis_par a;
    a.L = d == 0 ? boxd[0] : (d == 1 ? boxd[1] : boxd[2]);
    a.two_over_l = d == 0 ? box2i[0] : (d == 1 ? box2i[1] : box2i[2]);
    a.lim = d == 0 ? wlim[0] : (d == 1 ? wlim[1] : wlim[2]);
    return a;
}

__device__ __forceinline__ void check_moved(float4 p, float4 old, const md_kparams &kp,
                                            md_devstate *st)
{
    if (md_rsq_exact(p, old, kp) >= kp.rmaxdif) st->update = 1;
}

__device__ __forceinline__ void set_condition(const step_io &io)
{
    if (io.has_cond) {
        volatile md_devstate *vs = io.st;
        cudaGraphSetConditional(io.cond, vs->update ? 1u : 0u);
    }
}


inline thermo_par make_tp(const md_ctx *c, int energy)
{
    thermo_par tp;
    tp.t0 = c->temper_0;
    tp.tau = c->tau_t > 0 ? c->tau_t : 100.0;
    tp.ndf = md_ndf(c);
    tp.q_nh = tp.ndf * RGAS * tp.t0 * tp.tau * tp.tau;
    if (tp.q_nh <= 0) tp.q_nh = 1.0;
    tp.inv_ndfr = 1.0 / (tp.ndf * RGAS);
    tp.inv_q = 1.0 / tp.q_nh;
    tp.dt_tau = (double)c->dt / tp.tau;
    tp.berendsen = (c->enstype >= 1 && c->integrator == MD_LEAPFROG) ? 1 : 0;
    tp.npt = (c->enstype == 2 && c->batch) ? 1 : 0;
    tp.nh = (c->integrator == MD_NH) ? 1 : 0;
    tp.energy = energy;
    return tp;
}

inline step_io make_io(md_ctx *c, unsigned long long cond, int has_cond)
{
    step_io io;
    io.st = c->st;
    io.rec = c->rec;
    io.rep_hist = c->rep_hist;
    io.rec_cap = c->rec_cap;
    io.counter = &c->st->blocks_done;
    io.pos_old = c->pos_old;
    io.cond = (cudaGraphConditionalHandle)cond;
    io.has_cond = has_cond;
    return io;
}

}  // namespace

#endif
