/*
 * The reference's step loop (runGPU.cu:44-115, SimulationRun_CUDA) driven
 * through the reference-compatible entry points of libmdgpu_gb300
 * (md_gpu_compat.h), on a system read from a flat binary file.
 *
 *   compat_driver <input.bin> <output.bin> [vv]
 *
 * With "vv" the loop takes its velocity-Verlet form (runGPU.cu:73-97 with
 * vver = 1): integrate_pre, neighborlist, forces, energy, integrate_cor.
 *
 * input: int natom, ntype, lkspace, nmaxlist, enstype, nsteps, timprn;
 *        float box[3], rcutsq, reacf, alfa, skin, dt, temper_0;
 *        int itype[natom]; float charge[natom], pos[3 natom], vel[3 natom],
 *        mass[ntype], lj1[ntype^2], lj2[ntype^2]
 * output: float pos[3 natom], vel[3 natom], temper[nsteps]; then the
 *         charges after config_finish (unpacked from pos.w) [natom]
 */
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "md_gpu_compat.h"

template <class T>
static void rd(FILE *f, T *p, size_t n)
{
    if (fread(p, sizeof(T), n, f) != n) {
        fprintf(stderr, "short input\n");
        exit(2);
    }
}

int main(int argc, char **argv)
{
    if (argc != 3 && argc != 4) return 2;
    const bool vver = argc == 4;
    FILE *f = fopen(argv[1], "rb");
    if (!f) return 2;
    int hdr[7];
    float fh[9];
    rd(f, hdr, 7);
    rd(f, fh, 9);
    const int n = hdr[0], nt = hdr[1], nsteps = hdr[5];
    std::vector<int> itype(n);
    std::vector<float> q(n), pos(3 * n), vel(3 * n), mass(nt), lj1(nt * nt), lj2(nt * nt);
    rd(f, itype.data(), n);
    rd(f, q.data(), n);
    rd(f, pos.data(), 3 * n);
    rd(f, vel.data(), 3 * n);
    rd(f, mass.data(), nt);
    rd(f, lj1.data(), nt * nt);
    rd(f, lj2.data(), nt * nt);
    fclose(f);

    /* the structs as the reference's SimulationInit leaves them */
    config conf = {};
    conf.natom = n;
    conf.itype = itype.data();
    conf.box = make_float4(fh[0], fh[1], fh[2], 0.0f);
    conf.boxi = make_float4(1.0f / fh[0], 1.0f / fh[1], 1.0f / fh[2], 0.0f);
    std::vector<float4> p4(n), v4(n), f4(n);
    for (int i = 0; i < n; i++) {
        p4[i] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], q[i]);
        v4[i] = make_float4(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2], mass[itype[i]]);
        f4[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    conf.pos = p4.data();
    conf.vel = v4.data();
    conf.force = f4.data();
    ffield fld = {};
    fld.ntype = nt;
    fld.mass = mass.data();
    fld.lj1 = lj1.data();
    fld.lj2 = lj2.data();
    params pars = {};
    pars.timrun = nsteps - 1;
    pars.timprn = hdr[6];
    pars.lkspace = hdr[2];
    pars.nmaxlist = hdr[3];
    pars.rcutsq = fh[3];
    pars.reacf = fh[4];
    pars.alfa = fh[5];
    pars.skin = fh[6];
    integr integ = {};
    integ.enstype = hdr[4];
    integ.dt = fh[7];
    integ.temper_0 = fh[8];

    /* SimulationRun_CUDA */
    std::vector<float> temper(nsteps);
    gpu_struct *g_prop = gpu_properties_init(&conf);
    gpu_config *g_conf = config_init(&conf);
    checkCUDAError("config");
    gpu_ffield *g_fld = forces_init(&fld, &pars, &conf, g_prop, g_conf);
    gpu_nlist *g_nlist = neighborlist_init(&conf, g_prop, &pars, g_conf, &fld);
    gpu_integr *g_integ = integrate_init(&integ, g_prop, &conf);
    for (int t = 0; t <= pars.timrun; t++) {
        if (vver) integrate_pre(g_conf, g_integ, g_prop, &integ, &conf);
        neighborlist(g_prop, g_nlist, g_conf, &conf);
        forces(g_prop, g_nlist, g_conf, g_fld, &fld, &conf, &pars);
        if (t % pars.timprn == 0) energy(g_prop, g_nlist, g_conf, g_fld, &fld, &conf, &pars);
        if (vver)
            integrate_cor(g_conf, g_integ, g_prop, &integ, &conf);
        else
            integrate(g_conf, g_integ, g_prop, &integ, &conf);
        checkCUDAError("integrate");
        temper[t] = integ.temper;
    }
    config_DeviceToHost(&conf, g_conf, 1);
    for (int i = 0; i < n; i++) {
        pos[3 * i] = conf.pos[i].x;
        pos[3 * i + 1] = conf.pos[i].y;
        pos[3 * i + 2] = conf.pos[i].z;
        vel[3 * i] = conf.vel[i].x;
        vel[3 * i + 1] = conf.vel[i].y;
        vel[3 * i + 2] = conf.vel[i].z;
    }
    forces_finish(&fld, g_fld);
    config_finish(&conf, g_conf);
    integrate_finish(&integ, g_integ);
    neighborlist_finish(g_nlist);
    gpu_properties_finish(g_prop);
    for (int i = 0; i < n; i++) q[i] = conf.pos[i].w;

    FILE *o = fopen(argv[2], "wb");
    if (!o) return 2;
    fwrite(pos.data(), sizeof(float), 3 * n, o);
    fwrite(vel.data(), sizeof(float), 3 * n, o);
    fwrite(temper.data(), sizeof(float), nsteps, o);
    fwrite(q.data(), sizeof(float), n, o);
    fclose(o);
    return 0;
}
