/*
 * k_integrate.cu -- integrators and the FP64 thermodynamic reductions.
 *
 * Leapfrog (nve_leapfrog.cu:31-60, nvt_leapfrog_ber.cu:29-80):
 *   v <- (v + F dt/m') lambda,  x <- x + v dt,  x -= L trunc(2x/L)
 * with lambda = sqrt(1 + dt/tau (T0/T_prev - 1)) for Berendsen NVT
 * (integrator.cu:146-147, tau = 100 fs there) and 1 for NVE.  Positions and
 * velocities are FP64 here; the FP32 copy pos4 is refreshed in the same pass.
 * The kinetic energy is reduced in FP64, per block then by the last block to
 * finish in a fixed order (replacing the reference's single-block FP32 tree,
 * nvt_leapfrog_ber.cu:83-110, whose width is the block count).
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
#include "md_device.cuh"

namespace {

constexpr double RGAS = 8.314e-3;   /* kJ/mol/K, as integrator.cu:155 (1000/8.314) */

struct thermo_par {
    double t0, tau, q_nh;
    int ndf, berendsen, nh, energy;
};

/* Per-step bookkeeping buffers and the graph condition to set. */
struct step_io {
    md_devstate *st;
    double *partials;
    md_thermo *rec;
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

__device__ __forceinline__ double wrap(double x, double L)
{
    return x - L * trunc(x * 2.0 / L);
}

__device__ __forceinline__ void write_partials(double ke, double pe, double w, int energy,
                                               double *partials, double *sh)
{
    double a = block_sum(ke, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = a;
    if (energy) {
        double b = block_sum(pe, sh);
        double c = block_sum(w, sh);
        if (threadIdx.x == 0) {
            partials[gridDim.x + blockIdx.x] = b;
            partials[2 * gridDim.x + blockIdx.x] = c;
        }
    }
}

/* Fixed-order totals of the block partials, then (thread 0) temperature,
 * thermostat bookkeeping and the step record.  mode 0 leapfrog, 1 VV / NH,
 * 2 observe only (no step, the Berendsen reference temperature kept). */
__device__ void finalize(const md_kparams &kp, const thermo_par &tp, int mode, int npart,
                         const double *partials, md_devstate *st, md_thermo *rec, int rec_cap,
                         double *sh)
{
    double a = 0.0, b = 0.0, c = 0.0;
    for (int k = threadIdx.x; k < npart; k += blockDim.x) {
        a += __ldcg(partials + k);
        if (tp.energy) { b += __ldcg(partials + npart + k); c += __ldcg(partials + 2 * npart + k); }
    }
    double ke = block_sum(a, sh);
    double pe = tp.energy ? block_sum(b, sh) : 0.0;
    double w = tp.energy ? block_sum(c, sh) : 0.0;
    if (threadIdx.x != 0) return;
    volatile md_devstate *vs = st;
    double kt = RGAS * tp.t0;
    double lam = 1.0;
    if (mode == 0 && tp.berendsen) lam = sqrt(1.0 + kp.dt / tp.tau * (tp.t0 / vs->temper - 1.0));
    double xi = vs->xi, eta = vs->eta;
    if (mode == 1) {
        st->vscale = 1.0;
        if (tp.nh) {
            xi = vs->xi_a;
            eta = vs->eta_a;
            xi += 0.25 * kp.dt * (2.0 * ke - tp.ndf * kt) / tp.q_nh;
            double s2 = exp(-0.5 * kp.dt * xi);
            ke *= s2 * s2;
            eta += 0.5 * kp.dt * xi;
            xi += 0.25 * kp.dt * (2.0 * ke - tp.ndf * kt) / tp.q_nh;
            st->vscale = s2;
            st->xi = xi;
            st->eta = eta;
        }
    }
    double temper = 2.0 * ke / (tp.ndf * RGAS);
    st->ke = ke;
    if (tp.energy) { st->pe = pe; st->virial = w / 6.0; }
    /* observing the state does not move the Berendsen reference temperature:
     * the first step uses T = T0 (integrator.cu:77) */
    if (mode == 2) return;
    st->temper = temper;
    st->lambda = lam;
    long long step = vs->step;
    md_thermo r;
    r.step = step;
    r.ke = ke;
    r.temper = temper;
    r.pe = tp.energy ? pe : 0.0;
    r.virial = tp.energy ? w / 6.0 : 0.0;
    r.conserved = tp.energy ? ke + pe + (tp.nh ? 0.5 * tp.q_nh * xi * xi + tp.ndf * kt * eta : 0.0) : 0.0;
    r.xi = xi;
    r.lambda = lam;
    r.builds = vs->builds;
    r.flags = tp.energy ? 1 : 0;
    rec[step % rec_cap] = r;
    st->step = step + 1;
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

/* Leapfrog update + list check + KE partials; the last block finalises. */
__global__ void __launch_bounds__(256) k_leapfrog(md_kparams kp, thermo_par tp, step_io io,
                                                  double *x, double *v,
                                                  const double *__restrict__ mass, float4 *pos4,
                                                  const long long *__restrict__ f,
                                                  const float *__restrict__ epot,
                                                  const float *__restrict__ vir)
{
    __shared__ double sh[8];
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int P = kp.pitch;
    double lam = 1.0;
    if (tp.berendsen) lam = sqrt(1.0 + kp.dt / tp.tau * (tp.t0 / io.st->temper - 1.0));
    double ke = 0.0, pe = 0.0, w = 0.0;
    if (s < kp.n) {
        double m = mass[s], dtm = kp.dt / m;
        double xn[3];
        for (int d = 0; d < 3; d++) {
            double F = (double)f[d * P + s] * FX_INV;
            double vv = (v[d * P + s] + F * dtm) * lam;
            v[d * P + s] = vv;
            double xx = wrap(x[d * P + s] + vv * kp.dt, kp.boxd[d]);
            x[d * P + s] = xx;
            xn[d] = xx;
            ke += vv * vv;
        }
        ke *= 0.5 * m;
        float4 p = pos4[s];
        p = make_float4((float)xn[0], (float)xn[1], (float)xn[2], p.w);
        pos4[s] = p;
        check_moved(p, io.pos_old[s], kp, io.st);
        if (tp.energy) { pe = epot[s]; w = vir[s]; }
    }
    write_partials(ke, pe, w, tp.energy, io.partials, sh);
    if (md_last_block(io.counter)) {
        finalize(kp, tp, 0, gridDim.x, io.partials, io.st, io.rec, io.rec_cap, sh);
        if (threadIdx.x == 0) {
            set_condition(io);
            *io.counter = 0;
        }
    }
}

/* Velocity Verlet first half: thermostat half step (NH), half kick, drift,
 * list check; the last block sets the rebuild condition. */
__global__ void __launch_bounds__(256) k_vv_first(md_kparams kp, thermo_par tp, step_io io,
                                                  double *x, double *v,
                                                  const double *__restrict__ mass, float4 *pos4,
                                                  const long long *__restrict__ f)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int P = kp.pitch;
    md_devstate *st = io.st;
    double scale = st->vscale;
    if (tp.nh) {
        /* every thread evaluates the same scalar update; one thread stores it */
        double kt = RGAS * tp.t0, ke = st->ke, xi = st->xi, eta = st->eta;
        xi += 0.25 * kp.dt * (2.0 * ke - tp.ndf * kt) / tp.q_nh;
        double s1 = exp(-0.5 * kp.dt * xi);
        ke *= s1 * s1;
        eta += 0.5 * kp.dt * xi;
        xi += 0.25 * kp.dt * (2.0 * ke - tp.ndf * kt) / tp.q_nh;
        scale *= s1;
        if (s == 0) { st->xi_a = xi; st->eta_a = eta; }
    }
    if (s < kp.n) {
        double m = mass[s], hdtm = 0.5 * kp.dt / m;
        double xn[3];
        for (int d = 0; d < 3; d++) {
            double F = (double)f[d * P + s] * FX_INV;
            double vv = v[d * P + s] * scale + F * hdtm;
            v[d * P + s] = vv;
            double xx = wrap(x[d * P + s] + vv * kp.dt, kp.boxd[d]);
            x[d * P + s] = xx;
            xn[d] = xx;
        }
        float4 p = pos4[s];
        p = make_float4((float)xn[0], (float)xn[1], (float)xn[2], p.w);
        pos4[s] = p;
        check_moved(p, io.pos_old[s], kp, st);
    }
    if (md_last_block(io.counter)) {
        if (threadIdx.x == 0) {
            set_condition(io);
            *io.counter = 0;
        }
    }
}

/* Velocity Verlet second half kick and KE (PE, virial) partials; the last
 * block finalises.  kick = 0: observe the state only (pending NH scale
 * applied), mode 2. */
__global__ void __launch_bounds__(256) k_vv_second(md_kparams kp, thermo_par tp, int kick,
                                                   step_io io, double *v,
                                                   const double *__restrict__ mass,
                                                   const long long *__restrict__ f,
                                                   const float *__restrict__ epot,
                                                   const float *__restrict__ vir)
{
    __shared__ double sh[8];
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int P = kp.pitch;
    double ke = 0.0, pe = 0.0, w = 0.0;
    double scale = kick ? 1.0 : io.st->vscale;
    if (s < kp.n) {
        double m = mass[s], hdtm = 0.5 * kp.dt / m;
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
        finalize(kp, tp, kick ? 1 : 2, gridDim.x, io.partials, io.st, io.rec, io.rec_cap, sh);
        if (threadIdx.x == 0) *io.counter = 0;
    }
}

/* Original-order output: what 0 positions (3), 1 velocities (3, pending NH
 * scale applied), 2 forces + sum ff r^2 (4), 3 per-atom energy (1). */
__global__ void k_gather_out(md_kparams kp, int what, const md_devstate *st,
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
        double sc = st->vscale;
        for (int d = 0; d < 3; d++) out[3 * (size_t)o + d] = v[d * P + s] * sc;
    } else if (what == 2) {
        for (int d = 0; d < 3; d++) out[4 * (size_t)o + d] = (double)f[d * P + s] * FX_INV;
        out[4 * (size_t)o + 3] = vir[s];
    } else {
        out[o] = epot[s];
    }
}

/* Original-order input: what 0 positions (also refreshes pos4), 1 velocities. */
__global__ void k_scatter_in(md_kparams kp, int what, md_devstate *st,
                             const int *__restrict__ iperm, const double *__restrict__ in,
                             double *x, double *v, float4 *pos4)
{
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o == 0 && what == 1) st->vscale = 1.0;
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

thermo_par make_tp(const md_ctx *c, int energy)
{
    thermo_par tp;
    tp.t0 = c->temper_0;
    tp.tau = c->tau_t > 0 ? c->tau_t : 100.0;
    tp.ndf = 3 * c->n - 3;
    if (tp.ndf < 1) tp.ndf = 1;
    tp.q_nh = tp.ndf * RGAS * tp.t0 * tp.tau * tp.tau;
    if (tp.q_nh <= 0) tp.q_nh = 1.0;
    tp.berendsen = (c->enstype == 1 && c->integrator == MD_LEAPFROG) ? 1 : 0;
    tp.nh = (c->integrator == MD_NH) ? 1 : 0;
    tp.energy = energy;
    return tp;
}

step_io make_io(md_ctx *c, unsigned long long cond, int has_cond)
{
    step_io io;
    io.st = c->st;
    io.partials = c->partials;
    io.rec = c->rec;
    io.rec_cap = c->rec_cap;
    io.counter = &c->st->blocks_done;
    io.pos_old = c->pos_old;
    io.cond = (cudaGraphConditionalHandle)cond;
    io.has_cond = has_cond;
    return io;
}

}  // namespace

void launch_leapfrog(md_ctx *c, const md_kparams &kp, int energy, unsigned long long cond, int has_cond)
{
    int nb = (kp.n + 255) / 256;
    k_leapfrog<<<nb, 256, 0, c->stream>>>(kp, make_tp(c, energy), make_io(c, cond, has_cond), c->x,
                                          c->v, c->mass, c->pos4, c->f, c->epot, c->vir);
}

void launch_vv_first(md_ctx *c, const md_kparams &kp, unsigned long long cond, int has_cond)
{
    int nb = (kp.n + 255) / 256;
    k_vv_first<<<nb, 256, 0, c->stream>>>(kp, make_tp(c, 0), make_io(c, cond, has_cond), c->x,
                                          c->v, c->mass, c->pos4, c->f);
}

void launch_vv_second(md_ctx *c, const md_kparams &kp, int energy)
{
    int nb = (kp.n + 255) / 256;
    k_vv_second<<<nb, 256, 0, c->stream>>>(kp, make_tp(c, energy), 1, make_io(c, 0, 0), c->v,
                                           c->mass, c->f, c->epot, c->vir);
}

void launch_thermo_from_state(md_ctx *c, const md_kparams &kp, int energy)
{
    int nb = (kp.n + 255) / 256;
    k_vv_second<<<nb, 256, 0, c->stream>>>(kp, make_tp(c, energy), 0, make_io(c, 0, 0), c->v,
                                           c->mass, c->f, c->epot, c->vir);
}

void launch_gather_out(md_ctx *c, const md_kparams &kp, int what, void *dst)
{
    int nb = (kp.n + 255) / 256;
    k_gather_out<<<nb, 256, 0, c->stream>>>(kp, what, c->st, c->perm, c->x, c->v, c->f, c->vir,
                                            c->epot, (double *)dst);
}

void launch_scatter_in(md_ctx *c, const md_kparams &kp, int what, const void *src)
{
    int nb = (kp.n + 255) / 256;
    k_scatter_in<<<nb, 256, 0, c->stream>>>(kp, what, c->st, c->iperm, (const double *)src, c->x,
                                            c->v, c->pos4);
}
