/*
 * md_compat.cu -- the reference's host entry points of the step loop
 * (config.cu, gpu_properties.cu, forces.cu, neighborlist.cu, integrator.cu)
 * over the md_* C ABI; see include/md_gpu_compat.h for what each does.
 * Host code only: the work runs in the library's kernels.
 */
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "md_internal.h"
#include "../../include/md_gpu_compat.h"

namespace {

/* The one simulation of the process: the reference's structs it was
 * initialised with and the context made from them. */
struct compat_session {
    config *conf = nullptr;
    ffield *fld = nullptr;
    params *pars = nullptr;
    integr *integ = nullptr;
    md_ctx *ctx = nullptr;
    int energy_pending = 0;   /* energy() ran since the last integrate */
};
compat_session S;

/* The reference's error behaviour: report and leave the process. */
void die(const char *call, md_status s)
{
    char buf[512] = {0};
    md_last_error(S.ctx, buf, (int)sizeof(buf));
    fprintf(stderr, "md_gpu: %s: %s%s%s\n", call, md_status_string(s), buf[0] ? ": " : "", buf);
    exit(EXIT_FAILURE);
}

void check(const char *call, md_status s)
{
    if (s != MD_OK) die(call, s);
}

/* The charge of a packed pos.w = itype + 0.1 (q + 5), decoded as the
 * reference's kernels do (pair_forces.cu:44-45). */
float unpack_charge(float w)
{
    const float t = floorf(w);
    return (w - t) * 10.0f - 5.0f;
}

/* The context of the configuration the reference's structs describe. */
void create_context()
{
    config *c = S.conf;
    ffield *f = S.fld;
    params *p = S.pars;
    integr *in = S.integ;
    if (!c || !f || !p || !in) {
        fprintf(stderr, "md_gpu: integrate_init before config_init / forces_init\n");
        exit(EXIT_FAILURE);
    }
    if (in->enstype == 2) check("integrate_init", MD_ERR_UNSUPPORTED);
    const int n = c->natom;
    std::vector<float> q(n), pos(3 * (size_t)n), vel(3 * (size_t)n);
    for (int i = 0; i < n; i++) {
        q[i] = unpack_charge(c->pos[i].w);
        pos[3 * i] = c->pos[i].x;
        pos[3 * i + 1] = c->pos[i].y;
        pos[3 * i + 2] = c->pos[i].z;
        vel[3 * i] = c->vel[i].x;
        vel[3 * i + 1] = c->vel[i].y;
        vel[3 * i + 2] = c->vel[i].z;
    }
    std::vector<int> bonds(3 * (size_t)std::max(f->nbonds, 0)), angles(4 * (size_t)std::max(f->nangle, 0));
    for (int b = 0; b < f->nbonds; b++) {
        bonds[3 * b] = (int)f->iatn[b].w - 1;
        bonds[3 * b + 1] = (int)f->iatn[b].x - 1;
        bonds[3 * b + 2] = (int)f->iatn[b].y - 1;
    }
    for (int a = 0; a < f->nangle; a++) {
        angles[4 * a] = (int)f->iang[a].w - 1;
        angles[4 * a + 1] = (int)f->iang[a].x - 1;
        angles[4 * a + 2] = (int)f->iang[a].y - 1;
        angles[4 * a + 3] = (int)f->iang[a].z - 1;
    }
    md_system_desc d;
    memset(&d, 0, sizeof(d));
    d.natom = n;
    d.ntype = f->ntype;
    d.box[0] = c->box.x;
    d.box[1] = c->box.y;
    d.box[2] = c->box.z;
    d.itype = c->itype;
    d.charge = q.data();
    d.pos = pos.data();
    d.vel = vel.data();
    d.type_mass = f->mass;
    d.lj1 = f->lj1;
    d.lj2 = f->lj2;
    d.nbonds = f->nbonds;
    d.bonds = bonds.data();
    d.bnd1 = f->bnd1;
    d.bnd2 = f->bnd2;
    d.nangle = f->nangle;
    d.angles = angles.data();
    d.ang1 = f->ang1;
    d.ang2 = f->ang2;
    d.lkspace = p->lkspace;
    d.rcutsq = p->rcutsq;
    d.reacf = p->reacf;
    d.alfa = p->alfa;
    d.skin = p->skin;
    d.nmaxlist = p->nmaxlist;
    d.enstype = in->enstype;
    d.temper_0 = in->temper_0;
    d.dt = in->dt;
    d.tau_t = 100.0f;   /* the reference's thermostat constant (integrator.cu:146, 0.01 / fs) */
    d.integrator = MD_LEAPFROG;   /* the reference's active path (runGPU.cu:71) */
    check("integrate_init", md_create(&d, nullptr, &S.ctx));
}

void need_context(const char *call)
{
    if (!S.ctx) {
        fprintf(stderr, "md_gpu: %s before integrate_init\n", call);
        exit(EXIT_FAILURE);
    }
}

/* integ->temper and integ->Ke_sum[0] (kinetic energy), as the reference's
 * integrate() leaves them (integrator.cu:150-155). */
void thermo_to_integ(integr *integ)
{
    md_thermo t;
    check("integrate", md_get_thermo(S.ctx, &t));
    integ->temper = (float)t.temper;
    if (integ->Ke_sum) integ->Ke_sum[0] = (float)t.ke;
}

}  // namespace

md_ctx *md_compat_context() { return S.ctx; }

gpu_struct *gpu_properties_init(config *conf)
{
    gpu_struct *g = (gpu_struct *)calloc(1, sizeof(gpu_struct));
    cudaGetDeviceCount(&g->numdevices);
    cudaGetDevice(&g->thisdevice);
    g->prop = (cudaDeviceProp *)calloc(1, sizeof(cudaDeviceProp));
    cudaGetDeviceProperties(g->prop, g->thisdevice);
    g->block_size = 256;
    g->dimBlock = dim3(g->block_size, 1, 1);
    g->dimGrid = dim3((conf->natom + g->block_size - 1) / g->block_size, 1, 1);
    g->sharedMemSize = g->block_size * sizeof(float4);
    g->sum_dimGrid = dim3(1, 1, 1);
    g->sum_dimBlock = g->dimGrid;
    g->sum_sharedMemSize = g->dimGrid.x * sizeof(float);
    g->nblocks = g->dimGrid.x;
    return g;
}

void gpu_properties_finish(gpu_struct *g_prop)
{
    if (!g_prop) return;
    free(g_prop->prop);
    free(g_prop);
}

void checkCUDAError(const char *msg)
{
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) {
        fprintf(stderr, "Cuda error: %s: %s.\n", msg, cudaGetErrorString(err));
        exit(EXIT_FAILURE);
    }
}

gpu_config *config_init(config *conf)
{
    S.conf = conf;
    gpu_config *g = (gpu_config *)calloc(1, sizeof(gpu_config));
    const size_t bytes = sizeof(float4) * (size_t)conf->natom;
    if (cudaMalloc((void **)&g->pos, bytes) != cudaSuccess || cudaMalloc((void **)&g->vel, bytes) != cudaSuccess ||
        cudaMalloc((void **)&g->force, bytes) != cudaSuccess)
        check("config_init", MD_ERR_CUDA);
    for (int i = 0; i < conf->natom; i++)   /* config.cu:34 */
        conf->pos[i].w = (float)conf->itype[i] + 0.1f * (conf->pos[i].w + 5.0f);
    config_HostToDevice(conf, g);
    return g;
}

void config_HostToDevice(config *conf, gpu_config *g_conf)
{
    const size_t n = (size_t)conf->natom, bytes = sizeof(float4) * n;
    cudaMemcpy(g_conf->pos, conf->pos, bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(g_conf->vel, conf->vel, bytes, cudaMemcpyHostToDevice);
    if (conf->force) cudaMemcpy(g_conf->force, conf->force, bytes, cudaMemcpyHostToDevice);
    if (!S.ctx) return;
    std::vector<double> p(3 * n), v(3 * n);
    for (size_t i = 0; i < n; i++) {
        p[3 * i] = conf->pos[i].x;
        p[3 * i + 1] = conf->pos[i].y;
        p[3 * i + 2] = conf->pos[i].z;
        v[3 * i] = conf->vel[i].x;
        v[3 * i + 1] = conf->vel[i].y;
        v[3 * i + 2] = conf->vel[i].z;
    }
    check("config_HostToDevice", md_set_positions(S.ctx, p.data()));
    check("config_HostToDevice", md_set_velocities(S.ctx, v.data()));
}

void config_DeviceToHost(config *conf, gpu_config *g_conf, int icopy)
{
    const size_t n = (size_t)conf->natom, bytes = sizeof(float4) * n;
    if (S.ctx) {
        std::vector<double> b(4 * n);
        check("config_DeviceToHost", md_get_positions(S.ctx, b.data()));
        for (size_t i = 0; i < n; i++) {
            conf->pos[i].x = (float)b[3 * i];
            conf->pos[i].y = (float)b[3 * i + 1];
            conf->pos[i].z = (float)b[3 * i + 2];
        }
        cudaMemcpy(g_conf->pos, conf->pos, bytes, cudaMemcpyHostToDevice);
        if (icopy > 0) {
            check("config_DeviceToHost", md_get_velocities(S.ctx, b.data()));
            for (size_t i = 0; i < n; i++) {
                conf->vel[i].x = (float)b[3 * i];
                conf->vel[i].y = (float)b[3 * i + 1];
                conf->vel[i].z = (float)b[3 * i + 2];
            }
            cudaMemcpy(g_conf->vel, conf->vel, bytes, cudaMemcpyHostToDevice);
        }
        if (icopy > 1 && conf->force) {
            check("config_DeviceToHost", md_get_forces(S.ctx, b.data()));
            for (size_t i = 0; i < n; i++)
                conf->force[i] = make_float4((float)b[4 * i], (float)b[4 * i + 1], (float)b[4 * i + 2],
                                             (float)b[4 * i + 3]);
            cudaMemcpy(g_conf->force, conf->force, bytes, cudaMemcpyHostToDevice);
        }
        return;
    }
    cudaMemcpy(conf->pos, g_conf->pos, bytes, cudaMemcpyDeviceToHost);
    if (icopy > 0) cudaMemcpy(conf->vel, g_conf->vel, bytes, cudaMemcpyDeviceToHost);
    if (icopy > 1 && conf->force) cudaMemcpy(conf->force, g_conf->force, bytes, cudaMemcpyDeviceToHost);
}

void config_finish(config *conf, gpu_config *g_conf)
{
    config_DeviceToHost(conf, g_conf, 2);
    for (int i = 0; i < conf->natom; i++)   /* config.cu:46 */
        conf->pos[i].w = (conf->pos[i].w - (float)conf->itype[i]) * 10.0f - 5.0f;
    cudaFree(g_conf->pos);
    cudaFree(g_conf->vel);
    cudaFree(g_conf->force);
    free(g_conf);
    if (S.ctx) md_destroy(S.ctx);
    S = compat_session();
}

gpu_ffield *forces_init(ffield *fld, params *pars, config *conf, gpu_struct *, gpu_config *)
{
    S.fld = fld;
    S.pars = pars;
    S.conf = conf;
    return (gpu_ffield *)calloc(1, sizeof(gpu_ffield));
}

void forces(gpu_struct *, gpu_nlist *, gpu_config *, gpu_ffield *, ffield *, config *, params *)
{
    need_context("forces");
    check("forces", md_compute_forces(S.ctx, MD_TERM_ALL, 0));
    S.energy_pending = 0;
}

void energy(gpu_struct *, gpu_nlist *, gpu_config *, gpu_ffield *, ffield *, config *, params *)
{
    need_context("energy");
    /* forces with per-atom energies; the step's record takes them in the
     * next integrate (no observation of the state in between: in the middle
     * of a velocity-Verlet step it would move the thermostat) */
    md_kparams kp = md_make_kparams(S.ctx);
    launch_forces(S.ctx, kp, true, MD_TERM_ALL);
    if (cudaStreamSynchronize(S.ctx->stream) != cudaSuccess) check("energy", MD_ERR_CUDA);
    S.energy_pending = 1;
}

void forces_finish(ffield *, gpu_ffield *g_fld) { free(g_fld); }
void forces_HostToDevice(ffield *, gpu_ffield *) {}
void forces_DeviceToHost(ffield *, gpu_ffield *) {}

gpu_nlist *neighborlist_init(config *conf, gpu_struct *, params *pars, gpu_config *, ffield *fld)
{
    S.conf = conf;
    S.pars = pars;
    S.fld = fld;
    return (gpu_nlist *)calloc(1, sizeof(gpu_nlist));
}

void neighborlist(gpu_struct *, gpu_nlist *, gpu_config *, config *)
{
    need_context("neighborlist");
    check("neighborlist", md_update_neighbors(S.ctx, 0));
}

void neighborlist_finish(gpu_nlist *g_nlist) { free(g_nlist); }

gpu_integr *integrate_init(integr *integ, gpu_struct *g_prop, config *conf)
{
    S.integ = integ;
    S.conf = conf;
    integ->temper = integ->temper_0;   /* integrator.cu:77 */
    const int nb = g_prop ? (int)g_prop->dimGrid.x : 1;
    integ->Ke_sum = (float *)calloc((size_t)std::max(nb, 1), sizeof(float));
    integ->Wi_sum = (float *)calloc((size_t)std::max(nb, 1), sizeof(float));
    if (!S.ctx) create_context();
    return (gpu_integr *)calloc(1, sizeof(gpu_integr));
}

void integrate(gpu_config *, gpu_integr *, gpu_struct *, integr *integ, config *)
{
    need_context("integrate");
    check("integrate", md_integrate(S.ctx, S.energy_pending));
    S.energy_pending = 0;
    thermo_to_integ(integ);
}

void integrate_pre(gpu_config *, gpu_integr *, gpu_struct *, integr *, config *)
{
    need_context("integrate_pre");
    check("integrate_pre", md_integrate_pre(S.ctx));
}

void integrate_cor(gpu_config *, gpu_integr *, gpu_struct *, integr *integ, config *)
{
    need_context("integrate_cor");
    check("integrate_cor", md_integrate_cor(S.ctx, S.energy_pending));
    S.energy_pending = 0;
    thermo_to_integ(integ);
}

void integrate_HostToDevice(integr *, gpu_integr *, gpu_struct *) {}

void integrate_DeviceToHost(integr *integ, gpu_integr *, gpu_struct *)
{
    if (S.ctx) thermo_to_integ(integ);
}

void integrate_finish(integr *integ, gpu_integr *g_integ)
{
    free(integ->Ke_sum);
    free(integ->Wi_sum);
    integ->Ke_sum = integ->Wi_sum = nullptr;
    free(g_integ);
}
