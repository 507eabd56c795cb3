/*
 * ref_driver.cpp -- golden-vector generator: parses a case with the
 * reference's own SimulationInit (simulation.cu), then runs the reference's
 * kernels (emulated on the CPU) stage by stage and writes every intermediate
 * array to a binary record file.  TEST INFRASTRUCTURE.
 *
 *   ref_emu <case-dir> <case-name> <out.bin> [nsteps]
 *
 * Host glue that the reference keeps inside functions with kernel launches
 * (forces_init, neighborlist_init, integrate) is restated here, citing the
 * lines it follows; the kernels themselves are the reference's.
 */
#include "cuda_shim.h"
#include "ref_emu.h"

#include "simulation.h"
#include "runGPU.h"

#include <unistd.h>
#include <vector>

extern "C" void *ref_pad_malloc(size_t n) { return calloc(1, n * 8 + 4096); }

/* runGPU.h:33 -- never reached: the driver runs the stages itself. */
void SimulationRun_CUDA(params *, integr *, ffield *, config *) {}

static FILE *g_out;

static void put(const char *name, const char *dtype, const void *data, size_t count, size_t elsize)
{
    char nm[48] = {0}, dt[8] = {0};
    snprintf(nm, sizeof(nm), "%s", name);
    snprintf(dt, sizeof(dt), "%s", dtype);
    unsigned long long c = count;
    fwrite(nm, 1, 48, g_out);
    fwrite(dt, 1, 8, g_out);
    fwrite(&c, 8, 1, g_out);
    if (count) fwrite(data, elsize, count, g_out);
}
static void putf(const char *n, const float *d, size_t c) { put(n, "f4", d, c, 4); }
static void putu(const char *n, const unsigned *d, size_t c) { put(n, "u4", d, c, 4); }
static void puti(const char *n, const int *d, size_t c) { put(n, "i4", d, c, 4); }

int main(int argc, char **argv)
{
    if (argc < 4) { fprintf(stderr, "usage: ref_emu <dir> <name> <out.bin> [nsteps]\n"); return 2; }
    int nsteps = argc > 4 ? atoi(argv[4]) : 10;
    g_out = fopen(argv[3], "wb");
    if (!g_out) return 3;
    if (chdir(argv[1]) != 0) return 4;
    char name[80];
    snprintf(name, sizeof(name), "%s", argv[2]);
    simulation *sim = SimulationInit(name);
    params *pars = sim->pars;
    integr *integ = sim->integ;
    ffield *fld = sim->fld;
    config *conf = sim->conf;
    const int N = conf->natom;

    /* ---- parsed inputs ---- */
    float pv[12] = {pars->rcutsq, pars->reacf, pars->alfa, pars->skin, (float)pars->nmaxlist, integ->dt,
                    integ->temper_0, (float)pars->lkspace, (float)integ->enstype, (float)pars->timrun,
                    pars->rdel, 0.0f};
    putf("params", pv, 12);
    int fi[5] = {fld->ntype, fld->tbonds, fld->tangle, fld->nbonds, fld->nangle};
    puti("fld_counts", fi, 5);
    putf("mass", fld->mass, fld->ntype);
    putf("lj1", fld->lj1, 64);
    putf("lj2", fld->lj2, 64);
    putf("bnd1", fld->bnd1, 8);
    putf("bnd2", fld->bnd2, 8);
    putf("ang1", fld->ang1, 8);
    putf("ang2", fld->ang2, 8);
    std::vector<int> bonds(3 * fld->nbonds + 1), angles(4 * fld->nangle + 1);
    for (int i = 0; i < fld->nbonds; i++) {
        bonds[3 * i] = fld->iatn[i].w; bonds[3 * i + 1] = fld->iatn[i].x; bonds[3 * i + 2] = fld->iatn[i].y;
    }
    for (int i = 0; i < fld->nangle; i++) {
        angles[4 * i] = fld->iang[i].w; angles[4 * i + 1] = fld->iang[i].x;
        angles[4 * i + 2] = fld->iang[i].y; angles[4 * i + 3] = fld->iang[i].z;
    }
    puti("bonds", bonds.data(), 3 * fld->nbonds);
    puti("angles", angles.data(), 4 * fld->nangle);
    float bx[6] = {conf->box.x, conf->box.y, conf->box.z, conf->boxi.x, conf->boxi.y, conf->boxi.z};
    putf("box", bx, 6);
    puti("itype", conf->itype, N);
    putf("pos_in", (float *)conf->pos, 4 * (size_t)N);   /* w = charge as read */
    putf("vel_in", (float *)conf->vel, 4 * (size_t)N);   /* w = mass */

    /* ---- config_init packing, config.cu:33-35 ---- */
    for (int i = 0; i < N; i++) conf->pos[i].w = (float)(conf->itype[i]) + 0.1f * (conf->pos[i].w + 5.0f);
    putf("pos4", (float *)conf->pos, 4 * (size_t)N);

    /* ---- launch geometry, gpu_properties.cu:48-57 (block 256) ---- */
    const int pitch = ((N + 255) / 256) * 256;
    const unsigned nblk = (unsigned)(pitch / 256);

    /* ---- constants, forces.cu:80-110 and neighborlist.cu:35-48 ---- */
    RefConsts c;
    memset(&c, 0, sizeof(c));
    c.natom = N; c.ntype = fld->ntype; c.pitch = pitch;
    c.box = conf->box; c.boxi = conf->boxi;
    c.rcutsq = pars->rcutsq; c.reacf = pars->lkspace == 0 ? pars->reacf : 0.0f;
    for (int i = 0; i < 64; i++) { c.lj1[i] = fld->lj1[i]; c.lj2[i] = fld->lj2[i]; }
    if (pars->lkspace > 0) {
        c.palfa = pars->alfa * Pex;
        c.spiialfa = 2.0f / sqrtf(M_Pi) * pars->alfa;
        c.alfasq = -pars->alfa * pars->alfa / logf(2.0f);
        c.wolf = 0.0f;
        if (pars->lkspace == 1) {
            float ff = 1.0f / (1.0f + c.palfa * sqrt(pars->rcutsq));
            c.wolf = c.spiialfa * sqrtf(pars->rcutsq) + ((((A5 * ff + A4) * ff + A3) * ff + A2) * ff + A1) * ff;
            c.wolf *= exp2f(c.alfasq * pars->rcutsq) / sqrt(pars->rcutsq);
        }
    }
    for (int i = 0; i < 8; i++) { c.bnd1[i] = fld->bnd1[i]; c.bnd2[i] = fld->bnd2[i]; c.ang1[i] = fld->ang1[i]; c.ang2[i] = fld->ang2[i]; }
    c.dt = integ->dt; c.temper_0 = integ->temper_0; c.nblocks = nblk;
    c.rskinsq = pow(pars->skin + sqrt(pars->rcutsq), 2);
    c.rmaxdif = pars->skin * pars->skin / 4.0f;
    float kc[6] = {c.palfa, c.spiialfa, c.alfasq, c.wolf, c.rskinsq, c.rmaxdif};
    putf("consts", kc, 6);

    std::vector<float4> pos(conf->pos, conf->pos + N), vel(conf->vel, conf->vel + N);
    pos.resize(pitch); vel.resize(pitch);
    ref_set_consts(c, pos.data());

    /* ---- exclusions, neighborlist.cu:64-97 ---- */
    std::vector<uint4> excl(pitch);
    unsigned nat = (unsigned)N;
    for (int i = 0; i < N; i++) excl[i] = make_uint4(nat + 1, nat + 1, nat + 1, nat + 1);
    for (int it = 0; it < fld->nbonds; it++) {
        unsigned i = fld->iatn[it].x - 1, j = fld->iatn[it].y - 1;
        if (excl[i].x > nat) excl[i].x = j;
        else if (excl[i].y > nat) excl[i].y = j;
        else if (excl[i].z > nat) excl[i].z = j;
        else if (excl[i].w > nat) excl[i].w = j;
        if (excl[j].x > nat) excl[j].x = i;
        else if (excl[i].y > nat) excl[j].y = i;
        else if (excl[i].z > nat) excl[j].z = i;
        else if (excl[i].w > nat) excl[j].w = i;
    }
    putu("excl", (unsigned *)excl.data(), 4 * (size_t)N);

    /* ---- neighbour list ---- */
    const int nmax = pars->nmaxlist;
    std::vector<unsigned> nnlist((size_t)pitch * nmax + pitch, 0u), nnmax(pitch, 0u);
    std::vector<float4> pos_old(pitch);
    ref_nlist_nsquared(pos.data(), pos_old.data(), nnlist.data(), nnmax.data(), excl.data());
    unsigned mx = 0;
    for (int i = 0; i < N; i++) mx = nnmax[i] > mx ? nnmax[i] : mx;
    if ((int)mx > nmax) { fprintf(stderr, "list overflow %u > %d\n", mx, nmax); return 5; }
    putu("nnlist_max", nnmax.data(), N);
    {   /* rows i, first mx entries, row-major for compactness */
        std::vector<unsigned> rows((size_t)N * mx, 0xffffffffu);
        for (int i = 0; i < N; i++)
            for (unsigned k = 0; k < nnmax[i]; k++) rows[(size_t)i * mx + k] = nnlist[i + (size_t)pitch * k];
        putu("nnlist_rows", rows.data(), rows.size());
    }
    int chk0 = ref_nlist_check(pos.data(), pos_old.data());
    std::vector<float4> pos2 = pos;
    float half = sqrtf(c.rmaxdif);
    pos2[N / 2].x += 1.01f * half;   /* one atom beyond skin/2 */
    int chk1 = ref_nlist_check(pos2.data(), pos_old.data());
    std::vector<float4> pos3 = pos;
    pos3[N / 3].y += 0.99f * half;   /* one atom inside skin/2 */
    int chk2 = ref_nlist_check(pos3.data(), pos_old.data());
    int chk[3] = {chk0, chk1, chk2};
    puti("nlist_check", chk, 3);

    /* ---- forces, forces.cu:189-210 ---- */
    int kind = pars->lkspace == 0 ? 0 : 1;
    std::vector<float4> force(pitch);
    ref_pair(kind, force.data(), nnlist.data(), nnmax.data());
    putf("force_pair", (float *)force.data(), 4 * (size_t)N);
    std::vector<unsigned> blm(pitch, 0), alm(pitch, 0);
    std::vector<uint2> bl((size_t)pitch * 5);
    std::vector<uint4> al((size_t)pitch * 5);
    if (fld->nbonds > 0) {   /* forces.cu:118-134 */
        for (int it = 0; it < fld->nbonds; it++) {
            unsigned i = fld->iatn[it].x - 1, j = fld->iatn[it].y - 1, t = fld->iatn[it].w - 1;
            bl[i + (size_t)blm[i] * pitch] = make_uint2(j, t);
            bl[j + (size_t)blm[j] * pitch] = make_uint2(i, t);
            blm[i]++; blm[j]++;
        }
        ref_bonds(force.data(), bl.data(), blm.data());
        putf("force_bond", (float *)force.data(), 4 * (size_t)N);
    }
    if (fld->nangle > 0) {   /* forces.cu:147-173 */
        for (int it = 0; it < fld->nangle; it++) {
            unsigned i = fld->iang[it].x - 1, j = fld->iang[it].y - 1, k = fld->iang[it].z - 1, t = fld->iang[it].w - 1;
            al[i + (size_t)alm[i] * pitch] = make_uint4(0, j, k, t);
            al[j + (size_t)alm[j] * pitch] = make_uint4(1, i, k, t);
            al[k + (size_t)alm[k] * pitch] = make_uint4(0, j, i, t);
            alm[i]++; alm[j]++; alm[k]++;
        }
        ref_angles(force.data(), al.data(), alm.data());
        putf("force_angle", (float *)force.data(), 4 * (size_t)N);
    }
    putf("force_total", (float *)force.data(), 4 * (size_t)N);

    /* ---- integrators, one step each from the same state ---- */
    {
        std::vector<float4> p = pos, v = vel;
        ref_set_consts(c, p.data());
        ref_leapfrog_nve(p.data(), v.data(), force.data());
        putf("nve_pos", (float *)p.data(), 4 * (size_t)N);
        putf("nve_vel", (float *)v.data(), 4 * (size_t)N);
    }
    {
        std::vector<float4> p = pos, v = vel;
        std::vector<float> ke(nblk + 1, 0.0f);
        ref_set_consts(c, p.data());
        float tco = 0.01;   /* integrator.cu:146-147 with T = 0.9 T0 */
        float temper = 0.9f * integ->temper_0;
        float scale = sqrt(1.0f + integ->dt * tco * (integ->temper_0 / temper - 1.0f));
        ref_leapfrog_nvt(p.data(), v.data(), force.data(), scale, ke.data());
        putf("nvt_scale", &scale, 1);
        putf("nvt_pos", (float *)p.data(), 4 * (size_t)N);
        putf("nvt_vel", (float *)v.data(), 4 * (size_t)N);
        putf("nvt_ke_partials", ke.data(), nblk);
        ref_ke_sum(ke.data());
        ke[0] *= 0.5f;
        float tnew = ke[0] * 2.0f / (3.0f * (float)N - 3.0f) * 1000.0 / 8.314;
        float kt[2] = {ke[0], tnew};
        putf("nvt_ke_temper", kt, 2);
    }
    {
        std::vector<float4> p = pos, v = vel;
        ref_set_consts(c, p.data());
        ref_vv_pre(p.data(), v.data(), force.data());
        putf("vvpre_pos", (float *)p.data(), 4 * (size_t)N);
        putf("vvpre_vel", (float *)v.data(), 4 * (size_t)N);
        ref_vv_cor(v.data(), force.data());
        putf("vvcor_vel", (float *)v.data(), 4 * (size_t)N);
    }

    /* ---- the step loop, runGPU.cu:69-104 (timprn output omitted) ---- */
    {
        std::vector<float4> p = pos, v = vel, po = pos_old, fr(pitch);
        std::vector<float> ke(nblk + 1, 0.0f), temps(nsteps);
        ref_set_consts(c, p.data());
        float temper = integ->temper_0;   /* integrator.cu:77 */
        int builds = 1;
        for (int t = 0; t < nsteps; t++) {
            if (ref_nlist_check(p.data(), po.data()) == 1) {   /* neighborlist.cu:127-138 */
                ref_nlist_nsquared(p.data(), po.data(), nnlist.data(), nnmax.data(), excl.data());
                builds++;
            }
            ref_pair(kind, fr.data(), nnlist.data(), nnmax.data());
            if (fld->nbonds > 0) ref_bonds(fr.data(), bl.data(), blm.data());
            if (fld->nangle > 0) ref_angles(fr.data(), al.data(), alm.data());
            if (integ->enstype == 1) {   /* integrator.cu:145-155 */
                float tco = 0.01;
                float scale = sqrt(1.0f + integ->dt * tco * (integ->temper_0 / temper - 1.0f));
                ref_leapfrog_nvt(p.data(), v.data(), fr.data(), scale, ke.data());
                ref_ke_sum(ke.data());
                ke[0] *= 0.5f;
                temper = ke[0] * 2.0f / (3.0f * (float)N - 3.0f) * 1000.0 / 8.314;
            } else {
                ref_leapfrog_nve(p.data(), v.data(), fr.data());
            }
            temps[t] = temper;
        }
        putf("run_pos", (float *)p.data(), 4 * (size_t)N);
        putf("run_vel", (float *)v.data(), 4 * (size_t)N);
        putf("run_force", (float *)fr.data(), 4 * (size_t)N);
        putf("run_temps", temps.data(), nsteps);
        puti("run_builds", &builds, 1);
    }
    fclose(g_out);
    return 0;
}
