/*
 * k_integrate.cu -- integrators and the FP64 thermodynamic reductions.
 *
 * Leapfrog (nve_leapfrog.cu:31-60, nvt_leapfrog_ber.cu:29-80):
 *   v <- (v + F dt/m') lambda,  x <- x + v dt,  x -= L trunc(2x/L)
 * with lambda = sqrt(1 + dt/tau (T0/T_prev - 1)) for Berendsen NVT
 * (integrator.cu:146-147, tau = 100 fs there) and 1 for NVE.  Positions and
 * velocities are FP64 here; the FP32 copy pos4 is refreshed in the same pass.
 * The kinetic energy is reduced in FP64, per block then in one block in a
 * fixed order (replacing the reference's single-block FP32 tree,
 * nvt_leapfrog_ber.cu:83-110, whose width is the block count).
 *
 * Velocity Verlet: half kick + drift, forces, half kick.  Nose-Hoover adds a
 * thermostat half step on each side (single thermostat, Trotter splitting):
 *   xi += G dt/4;  v *= exp(-xi dt/2);  eta += xi dt/2;  xi += G dt/4,
 *   G = (2 KE - ndf k T0) / Q,  Q = ndf k T0 tau^2,
 * with the conserved quantity KE + PE + Q xi^2/2 + ndf k T0 eta.
 */
#include "md_internal.h"

namespace {

constexpr double RGAS = 8.314e-3;   /* kJ/mol/K, as integrator.cu:155 (1000/8.314) */

struct thermo_par {
    double t0, tau, q_nh;
    int ndf, berendsen, nh, energy;
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

__global__ void __launch_bounds__(256) k_leapfrog(md_kparams kp, thermo_par tp,
                                                  const md_devstate *st, double *x, double *v,
                                                  const double *__restrict__ mass, float4 *pos4,
                                                  const long long *__restrict__ f,
                                                  const float *__restrict__ epot,
                                                  const float *__restrict__ vir, double *partials)
{
    __shared__ double sh[8];
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int P = kp.pitch;
    double lam = 1.0;
    if (tp.berendsen) lam = sqrt(1.0 + kp.dt / tp.tau * (tp.t0 / st->temper - 1.0));
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
        pos4[s] = make_float4((float)xn[0], (float)xn[1], (float)xn[2], p.w);
        if (tp.energy) { pe = epot[s]; w = vir[s]; }
    }
    double a = block_sum(ke, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = a;
    if (tp.energy) {
        double b = block_sum(pe, sh);
        double c = block_sum(w, sh);
        if (threadIdx.x == 0) {
            partials[gridDim.x + blockIdx.x] = b;
            partials[2 * gridDim.x + blockIdx.x] = c;
        }
    }
}

/* Velocity Verlet first half: thermostat half step (NH), half kick, drift. */
__global__ void __launch_bounds__(256) k_vv_first(md_kparams kp, thermo_par tp, md_devstate *st,
                                                  double *x, double *v,
                                                  const double *__restrict__ mass, float4 *pos4,
                                                  const long long *__restrict__ f)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int P = kp.pitch;
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
    if (s >= kp.n) return;
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
    pos4[s] = make_float4((float)xn[0], (float)xn[1], (float)xn[2], p.w);
}

/* Velocity Verlet second half kick and the block partials of KE (and PE,
 * virial); scale != 1 only for the state read-out kernel below. */
__global__ void __launch_bounds__(256) k_vv_second(md_kparams kp, thermo_par tp, int kick,
                                                   const md_devstate *st, double *v,
                                                   const double *__restrict__ mass,
                                                   const long long *__restrict__ f,
                                                   const float *__restrict__ epot,
                                                   const float *__restrict__ vir,
                                                   double *partials)
{
    __shared__ double sh[8];
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int P = kp.pitch;
    double ke = 0.0, pe = 0.0, w = 0.0;
    double scale = kick ? 1.0 : st->vscale;
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
    double a = block_sum(ke, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = a;
    if (tp.energy) {
        double b = block_sum(pe, sh);
        double c = block_sum(w, sh);
        if (threadIdx.x == 0) {
            partials[gridDim.x + blockIdx.x] = b;
            partials[2 * gridDim.x + blockIdx.x] = c;
        }
    }
}

/* One block: fixed-order sums of the partials, temperature, thermostat
 * bookkeeping and the step record.  mode 0 leapfrog, 1 VV / NH, 2 observe
 * only (no step). */
__global__ void __launch_bounds__(256) k_finalize(md_kparams kp, thermo_par tp, int mode,
                                                  int npart, const double *__restrict__ partials,
                                                  md_devstate *st, md_thermo *rec, int rec_cap)
{
    __shared__ double sh[8];
    double a = 0.0, b = 0.0, c = 0.0;
    for (int k = threadIdx.x; k < npart; k += blockDim.x) {
        a += partials[k];
        if (tp.energy) { b += partials[npart + k]; c += partials[2 * npart + k]; }
    }
    double ke = block_sum(a, sh);
    double pe = tp.energy ? block_sum(b, sh) : 0.0;
    double w = tp.energy ? block_sum(c, sh) : 0.0;
    if (threadIdx.x != 0) return;
    double kt = RGAS * tp.t0;
    double lam = 1.0;
    if (mode == 0 && tp.berendsen) lam = sqrt(1.0 + kp.dt / tp.tau * (tp.t0 / st->temper - 1.0));
    double xi = st->xi, eta = st->eta;
    if (mode == 1) {
        st->vscale = 1.0;
        if (tp.nh) {
            xi = st->xi_a;
            eta = st->eta_a;
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
    long long step = st->step;
    md_thermo r;
    r.step = step;
    r.ke = ke;
    r.temper = temper;
    r.pe = tp.energy ? pe : 0.0;
    r.virial = tp.energy ? w / 6.0 : 0.0;
    r.conserved = tp.energy ? ke + pe + (tp.nh ? 0.5 * tp.q_nh * xi * xi + tp.ndf * kt * eta : 0.0) : 0.0;
    r.xi = xi;
    r.lambda = lam;
    r.builds = st->builds;
    r.flags = tp.energy ? 1 : 0;
    rec[step % rec_cap] = r;
    st->step = step + 1;
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

}  // namespace

void launch_leapfrog(md_ctx *c, const md_kparams &kp, int energy)
{
    thermo_par tp = make_tp(c, energy);
    int nb = (kp.n + 255) / 256;
    k_leapfrog<<<nb, 256, 0, c->stream>>>(kp, tp, c->st, c->x, c->v, c->mass, c->pos4, c->f,
                                          c->epot, c->vir, c->partials);
    k_finalize<<<1, 256, 0, c->stream>>>(kp, tp, 0, nb, c->partials, c->st, c->rec, c->rec_cap);
}

void launch_vv_first(md_ctx *c, const md_kparams &kp)
{
    thermo_par tp = make_tp(c, 0);
    int nb = (kp.n + 255) / 256;
    k_vv_first<<<nb, 256, 0, c->stream>>>(kp, tp, c->st, c->x, c->v, c->mass, c->pos4, c->f);
}

void launch_vv_second(md_ctx *c, const md_kparams &kp, int energy)
{
    thermo_par tp = make_tp(c, energy);
    int nb = (kp.n + 255) / 256;
    k_vv_second<<<nb, 256, 0, c->stream>>>(kp, tp, 1, c->st, c->v, c->mass, c->f, c->epot,
                                           c->vir, c->partials);
    k_finalize<<<1, 256, 0, c->stream>>>(kp, tp, 1, nb, c->partials, c->st, c->rec, c->rec_cap);
}

void launch_thermo_from_state(md_ctx *c, const md_kparams &kp, int energy)
{
    thermo_par tp = make_tp(c, energy);
    int nb = (kp.n + 255) / 256;
    k_vv_second<<<nb, 256, 0, c->stream>>>(kp, tp, 0, c->st, c->v, c->mass, c->f, c->epot,
                                           c->vir, c->partials);
    k_finalize<<<1, 256, 0, c->stream>>>(kp, tp, 2, nb, c->partials, c->st, c->rec, c->rec_cap);
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
