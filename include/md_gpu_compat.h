/*
 * md_gpu_compat.h -- the reference's own host entry points of the step loop,
 * with its names, C++ signatures and struct layouts, implemented over
 * libmdgpu_gb300 (md_compat.cu).
 *
 * A program written against the reference (its main loop SimulationRun_CUDA,
 * runGPU.cu:44-115, its input parsers in simulation.cu and its printing
 * helpers in prints.cu) links against this library in place of the
 * reference's config.cu, gpu_properties.cu, forces.cu, neighborlist.cu and
 * integrator.cu.  The mangled names match the reference's, because the
 * functions have C++ linkage and the typedef names and member layouts of the
 * structs below are the reference's (simulation.h:51-122, config.h:32-39,
 * forces.h:32-42, neighborlist.h:29-38, integrator.h:32-48,
 * gpu_properties.h:32-44).  The caller fills config, ffield, params and
 * integr as the reference's SimulationInit does (charges in pos.w before
 * config_init, masses x 1e4 in vel.w, 1-based bond and angle atoms in
 * ffield.iatn / ffield.iang).
 *
 * What each call does here:
 *   gpu_properties_init   device properties (block size 256, grid over the atoms)
 *   config_init           packs pos.w = itype + 0.1 (q + 5) (config.cu:34) and
 *                         keeps device copies of pos, vel, force
 *   forces_init, neighborlist_init, integrate_init
 *                         record the inputs; integrate_init (the last of the
 *                         reference's init calls) creates the md_ctx: list,
 *                         forces and thermodynamic state of the configuration
 *   neighborlist          md_update_neighbors (skin/2 check, rebuild)
 *   forces                md_compute_forces (pair, bonds, angles)
 *   energy                the same with energies (the reference's is empty);
 *                         the next integrate puts them in its record
 *   integrate             md_integrate; integ->temper and integ->Ke_sum[0]
 *                         (kinetic energy) are updated as the reference does
 *   integrate_pre / _cor  md_integrate_pre / md_integrate_cor
 *   config_HostToDevice   uploads conf->pos / vel into the context
 *   config_DeviceToHost   positions (icopy >= 0), velocities (>= 1) and
 *                         forces with sum ff r^2 in w (>= 2) back into conf
 *   *_finish              free; config_finish unpacks pos.w back to charges
 *
 * One simulation per process (the reference keeps its device state in
 * __constant__ memory and is not re-entrant either).  Errors behave as in
 * the reference: the call prints a message and exits the process
 * (checkCUDAError, gpu_properties.cu:75-81); the md_* C ABI returns status
 * codes instead.  NPT (enstype 2) is not implemented.
 */
#ifndef MD_GPU_COMPAT_H
#define MD_GPU_COMPAT_H

#include <cuda_runtime.h>
#include <vector_types.h>

/* --- simulation.h --- */
typedef struct {
    int natom;
    int *itype;    /* 0-based */
    float4 box;
    float4 boxi;
    float4 *pos;   /* x, y, z and the charge (packed with the type by config_init) */
    float4 *vel;   /* vx, vy, vz and the mass x 1e4 */
    float4 *force; /* fx, fy, fz and sum ff r^2 */
} config;

typedef struct {
    int ntype;
    int *nt;
    char **name;
    float *mass;
    float *charge;
    float *lj1;    /* ntype x ntype, row stride ntype */
    float *lj2;
    float *bnd1;
    float *bnd2;
    float *ang1;
    float *ang2;
    int tbonds;
    int tangle;
    int nrigid;
    int nbonds;
    int nangle;
    int nmaxbond;
    unsigned int *bndlist_max;
    uint2 *bndlist;
    uint4 *iatn;   /* bonds: x = i, y = j, w = type (1-based) */
    unsigned int *anglist_max;
    uint4 *anglist;
    uint4 *iang;   /* angles: x = i, y = j (centre), z = k, w = type (1-based) */
} ffield;

typedef struct {
    int timeq;
    int timrun;
    int timprn;
    float rcutsq;
    float reacf;
    int lkspace;
    int kmax;
    float alfa;
    float skin;
    int nmaxlist;
    float rdel;
} params;

typedef struct {
    float4 tdm;
    float4 energ_nonbond;
    float4 energ_bonded;
} thermodyn;

typedef struct {
    char *ensemble;
    int enstype;   /* 0 NVE, 1 NVT (Berendsen leapfrog / Nose-Hoover VV), 2 NPT */
    float dt;
    float temper_0;
    float tcons;
    float press_0;
    float pcons;
    float temper;
    float *Ke_sum;
    float *Wi_sum;
    float *Ke_total;
    float *Wi_total;
    thermodyn *therm;
} integr;

/* --- config.h, forces.h, neighborlist.h, integrator.h, gpu_properties.h --- */
typedef struct {
    float4 *pos;
    float4 *vel;
    float4 *force;
} gpu_config;

typedef struct {
    float something;
    uint2 *bndlist;
    unsigned int *bndlist_max;
    uint4 *anglist;
    unsigned int *anglist_max;
} gpu_ffield;

typedef struct {
    float4 *pos_old;
    unsigned int *nnlist;
    unsigned int *nnlist_max;
    uint4 *excl;
    int *update;
} gpu_nlist;

typedef struct {
    float4 tdm;
    float4 energ_nonbond;
    float4 energ_bonded;
} gpu_thermodyn;

typedef struct {
    float2 st;
    float2 sp;
    float *Ke_sum;
    float *Wi_sum;
    float *Ke_total;
    float *Wi_total;
    gpu_thermodyn *g_therm;
} gpu_integr;

typedef struct {
    int numdevices;
    int thisdevice;
    int block_size;
    dim3 dimGrid;
    dim3 dimBlock;
    size_t sharedMemSize;
    dim3 sum_dimGrid;
    dim3 sum_dimBlock;
    size_t sum_sharedMemSize;
    unsigned int nblocks;
    cudaDeviceProp *prop;
} gpu_struct;

/* gpu_properties.h:46-48 */
gpu_struct *gpu_properties_init(config *conf);
void gpu_properties_finish(gpu_struct *g_prop);
void checkCUDAError(const char *msg);
/* config.h:41-44 */
gpu_config *config_init(config *conf);
void config_finish(config *conf, gpu_config *g_conf);
void config_HostToDevice(config *conf, gpu_config *g_conf);
void config_DeviceToHost(config *conf, gpu_config *g_conf, int icopy);
/* forces.h:44-50 */
gpu_ffield *forces_init(ffield *fld, params *pars, config *conf, gpu_struct *g_prop, gpu_config *g_conf);
void forces(gpu_struct *g_prop, gpu_nlist *g_nlist, gpu_config *g_conf, gpu_ffield *g_fld, ffield *fld,
            config *conf, params *pars);
void forces_finish(ffield *fld, gpu_ffield *g_fld);
void forces_HostToDevice(ffield *fld, gpu_ffield *g_fld);
void forces_DeviceToHost(ffield *fld, gpu_ffield *g_fld);
void energy(gpu_struct *g_prop, gpu_nlist *g_nlist, gpu_config *g_conf, gpu_ffield *g_fld, ffield *fld,
            config *conf, params *pars);
/* neighborlist.h:40-42 */
gpu_nlist *neighborlist_init(config *conf, gpu_struct *g_prop, params *pars, gpu_config *g_conf, ffield *fld);
void neighborlist(gpu_struct *g_prop, gpu_nlist *g_nlist, gpu_config *g_conf, config *conf);
void neighborlist_finish(gpu_nlist *g_nlist);
/* integrator.h:50-56 */
gpu_integr *integrate_init(integr *integ, gpu_struct *g_prop, config *conf);
void integrate_finish(integr *integ, gpu_integr *g_integ);
void integrate(gpu_config *g_conf, gpu_integr *g_integ, gpu_struct *g_prop, integr *integ, config *conf);
void integrate_pre(gpu_config *g_conf, gpu_integr *g_integ, gpu_struct *g_prop, integr *integ, config *conf);
void integrate_cor(gpu_config *g_conf, gpu_integr *g_integ, gpu_struct *g_prop, integr *integ, config *conf);
void integrate_HostToDevice(integr *integ, gpu_integr *g_integ, gpu_struct *g_prop);
void integrate_DeviceToHost(integr *integ, gpu_integr *g_integ, gpu_struct *g_prop);

/* The context behind the compat calls (NULL before integrate_init), for
 * callers that mix them with the md_* C ABI. */
struct md_ctx;
md_ctx *md_compat_context();

#endif
