/*
 * md_api.cu -- host side of libmdgpu_gb300: input parsing, context set-up,
 * the CUDA-graph step driver and the C ABI declared in include/md_gpu.h.
 *
 * Reference counterparts: SimulationInit / FFieldInput / ConfigInput
 * (simulation.cu:40-316), config_init (config.cu:22-40), forces_init
 * (forces.cu:75-186), neighborlist_init (neighborlist.cu:30-107),
 * integrate_init (integrator.cu:47-97) and the step loop of
 * SimulationRun_CUDA (runGPU.cu:69-104).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "md_internal.h"

namespace {

std::string g_last_error;

/* ---------------- input files (own restatement of simulation.cu) ---------------- */

struct parsed_run {
    md_system_desc d;
    std::vector<int> itype, bonds, angles;
    std::vector<float> charge, pos, vel, mass, lj1, lj2, bnd1, bnd2, ang1, ang2;
    std::vector<std::string> names;   /* per type, from the .fld */
    int timprn = 1;
    float rdel = 0.02f;
    float press0 = 1.0f, tau_p = 1000.0f, beta = 4.5e-5f;   /* NPT: bar, fs, 1/bar */
    float pme_spacing = 0.0f;   /* lkspace 2: PME grid spacing, A (0: real-space term only) */
};

/* .inp (simulation.cu:58-105): label tokens skipped; reacf and alfa derived
 * with the reference's float/double mix; extension lines after rdel. */
md_status parse_inp(const char *path, parsed_run &r)
{
    FILE *fin = fopen(path, "r");
    if (!fin) return MD_ERR_IO;
    char lab[256], ens[64];
    md_system_desc &d = r.d;
    int timeq, timrun;
    float rc;
    md_status st = MD_ERR_PARSE;
    d.tau_t = 100.0f;
    d.integrator = MD_LEAPFROG;
    if (fscanf(fin, "%255s %63s", lab, ens) != 2) goto out;
    d.enstype = 0;
    if (!strcmp(ens, "nvt")) {
        d.enstype = 1;
        if (fscanf(fin, "%255s %f", lab, &d.temper_0) != 2) goto out;
    } else if (!strcmp(ens, "npt")) {   /* simulation.cu:71-75: T0 and P0 */
        d.enstype = 2;
        if (fscanf(fin, "%255s %f %f", lab, &d.temper_0, &r.press0) != 3) goto out;
    }
    if (fscanf(fin, "%255s %d %d %d %f", lab, &timeq, &timrun, &r.timprn, &d.dt) != 5) goto out;
    if (fscanf(fin, "%255s %f %d", lab, &rc, &d.lkspace) != 3) goto out;
    if (d.lkspace == 0) {
        float eps;
        if (fscanf(fin, "%255s %f", lab, &eps) != 2) goto out;
        float num = 2.0f * (eps - 1.0f) / (2.0f * eps + 1.0f);
        d.reacf = (float)((double)num / pow((double)rc, 3.0));
    } else if (d.lkspace == 1) {
        if (fscanf(fin, "%255s %f", lab, &d.alfa) != 2) goto out;
    } else {
        int kmax;
        if (fscanf(fin, "%255s %d", lab, &kmax) != 2) goto out;
        d.alfa = (float)(3.09 / (double)rc);
    }
    d.rcutsq = rc * rc;
    if (fscanf(fin, "%255s %f %d", lab, &d.skin, &d.nmaxlist) != 3) goto out;
    if (fscanf(fin, "%255s %f", lab, &r.rdel) != 2) goto out;
    {
        char val[64];
        while (fscanf(fin, "%255s %63s", lab, val) == 2) {
            if (!strcmp(lab, "tau_t:")) d.tau_t = strtof(val, nullptr);
            else if (!strcmp(lab, "tau_p:")) r.tau_p = strtof(val, nullptr);
            else if (!strcmp(lab, "compressibility:")) r.beta = strtof(val, nullptr);
            else if (!strcmp(lab, "pme_spacing:")) r.pme_spacing = strtof(val, nullptr);
            else if (!strcmp(lab, "integrator:"))
                d.integrator = !strcmp(val, "vv") ? MD_VV : (!strcmp(val, "nh") ? MD_NH : MD_LEAPFROG);
        }
    }
    st = MD_OK;
out:
    fclose(fin);
    return st;
}

/* .fld (simulation.cu:144-264). */
md_status parse_fld(const char *path, parsed_run &r)
{
    FILE *fin = fopen(path, "r");
    if (!fin) return MD_ERR_IO;
    char lab[256], name[64], form[64];
    int ntype, iaux, cnt, nvdw, i, j;
    float a, b;
    md_status st = MD_ERR_PARSE;
    if (fscanf(fin, "%255s %d", lab, &ntype) != 2 || ntype < 1 || ntype > MD_MAXTYPE) goto out;
    r.mass.assign(ntype, 0.0f);
    r.lj1.assign(ntype * ntype, 0.0f);
    r.lj2.assign(ntype * ntype, 0.0f);
    for (int t = 0; t < ntype; t++) {
        float m, q;
        if (fscanf(fin, "%d %d", &iaux, &cnt) != 2) goto out;
        if (fscanf(fin, "%63s %f %f", name, &m, &q) != 3) goto out;
        r.mass[t] = (float)((double)m * 10000.0);
        r.names.push_back(name);
    }
    if (fscanf(fin, "%255s %d", lab, &nvdw) != 2) goto out;
    for (int t = 0; t < nvdw; t++) {
        if (fscanf(fin, "%d %d %63s %f %f", &i, &j, form, &a, &b) != 5) goto out;
        i--; j--;
        if (i < 0 || j < 0 || i >= ntype || j >= ntype) goto out;
        float l1, l2;
        if (!strcmp(form, "LJ")) {
            l1 = (float)((double)(12.0f * 4.0f * b) * pow((double)a, 12.0));
            l2 = (float)((double)(6.0f * 4.0f * b) * pow((double)a, 6.0));
        } else if (!strcmp(form, "12-6")) {
            l1 = 12.0f * a;
            l2 = 6.0f * b;
        } else {
            continue;
        }
        r.lj1[i * ntype + j] = r.lj1[j * ntype + i] = l1;
        r.lj2[i * ntype + j] = r.lj2[j * ntype + i] = l2;
    }
    int tb, ta, nb, na;
    if (fscanf(fin, "%255s %d", lab, &tb) != 2 || tb < 0 || tb > MD_MAXTYPE) goto out;
    r.bnd1.assign(MD_MAXTYPE, 0.0f);
    r.bnd2.assign(MD_MAXTYPE, 0.0f);
    for (int t = 0; t < tb; t++) {
        if (fscanf(fin, "%d %f %f", &iaux, &r.bnd1[t], &r.bnd2[t]) != 3) goto out;
        r.bnd1[t] *= 2.0f;
    }
    if (fscanf(fin, "%255s %d", lab, &ta) != 2 || ta < 0 || ta > MD_MAXTYPE) goto out;
    r.ang1.assign(MD_MAXTYPE, 0.0f);
    r.ang2.assign(MD_MAXTYPE, 0.0f);
    for (int t = 0; t < ta; t++) {
        if (fscanf(fin, "%d %f %f", &iaux, &r.ang1[t], &r.ang2[t]) != 3) goto out;
        r.ang1[t] *= 2.0f;
        r.ang2[t] *= 3.1415927f / 180.0f;
    }
    if (fscanf(fin, "%255s %d", lab, &nb) != 2 || nb < 0) goto out;
    r.bonds.resize(3 * (size_t)nb);
    for (int t = 0; t < nb; t++) {
        int ty, bi, bj;
        if (fscanf(fin, "%d %d %d %d", &iaux, &ty, &bi, &bj) != 4) goto out;
        r.bonds[3 * t] = ty - 1; r.bonds[3 * t + 1] = bi - 1; r.bonds[3 * t + 2] = bj - 1;
    }
    if (fscanf(fin, "%255s %d", lab, &na) != 2 || na < 0) goto out;
    r.angles.resize(4 * (size_t)na);
    for (int t = 0; t < na; t++) {
        int ty, ai, aj, ak;
        if (fscanf(fin, "%d %d %d %d %d", &iaux, &ty, &ai, &aj, &ak) != 5) goto out;
        r.angles[4 * t] = ty - 1; r.angles[4 * t + 1] = ai - 1;
        r.angles[4 * t + 2] = aj - 1; r.angles[4 * t + 3] = ak - 1;
    }
    r.d.ntype = ntype;
    r.d.nbonds = nb;
    r.d.nangle = na;
    st = MD_OK;
out:
    fclose(fin);
    return st;
}

/* .cfg (simulation.cu:278-316). */
md_status parse_cfg(const char *path, parsed_run &r)
{
    FILE *fin = fopen(path, "r");
    if (!fin) return MD_ERR_IO;
    int n, cftyp, iaux;
    md_status st = MD_ERR_PARSE;
    if (fscanf(fin, "%d %d", &n, &cftyp) != 2 || n <= 0) goto out;
    if (fscanf(fin, "%f %f %f", &r.d.box[0], &r.d.box[1], &r.d.box[2]) != 3) goto out;
    r.itype.resize(n);
    r.charge.resize(n);
    r.pos.assign(3 * (size_t)n, 0.0f);
    r.vel.assign(3 * (size_t)n, 0.0f);
    for (int i = 0; i < n; i++) {
        if (fscanf(fin, "%d %d %f", &iaux, &r.itype[i], &r.charge[i]) != 3) goto out;
        r.itype[i] -= 1;
        if (fscanf(fin, "%f %f %f", &r.pos[3 * i], &r.pos[3 * i + 1], &r.pos[3 * i + 2]) != 3) goto out;
        if (cftyp > 0)
            if (fscanf(fin, "%f %f %f", &r.vel[3 * i], &r.vel[3 * i + 1], &r.vel[3 * i + 2]) != 3) goto out;
    }
    r.d.natom = n;
    st = MD_OK;
out:
    fclose(fin);
    return st;
}

/* ---------------- derived constants ---------------- */

/* forces.cu:97-110 (C++: sqrt of a float is the float overload). */
void wolf_consts(float alfa, float rcutsq, float out[4])
{
    const float P = 0.3275911f, A1 = 0.254829592f, A2 = -0.284496736f, A3 = 1.421413741f,
                A4 = -1.453152027f, A5 = 1.061405429f;
    float palfa = alfa * P;
    float spiialfa = 2.0f / sqrtf(3.1415927f) * alfa;
    float alfasq = -alfa * alfa / logf(2.0f);
    float ff = 1.0f / (1.0f + palfa * sqrtf(rcutsq));
    float wolf = spiialfa * sqrtf(rcutsq) + ((((A5 * ff + A4) * ff + A3) * ff + A2) * ff + A1) * ff;
    wolf *= exp2f(alfasq * rcutsq) / sqrtf(rcutsq);
    out[0] = palfa; out[1] = spiialfa; out[2] = alfasq; out[3] = wolf;
}

/* 3-D Hilbert index (Skilling, AIP Conf. Proc. 707 (2004) 381). */
unsigned long long hilbert3(unsigned x, unsigned y, unsigned z, int bits)
{
    unsigned X[3] = {x, y, z};
    unsigned M = 1u << (bits - 1), P, Q, t;
    for (Q = M; Q > 1; Q >>= 1) {
        P = Q - 1;
        for (int i = 0; i < 3; i++) {
            if (X[i] & Q) X[0] ^= P;
            else { t = (X[0] ^ X[i]) & P; X[0] ^= t; X[i] ^= t; }
        }
    }
    for (int i = 1; i < 3; i++) X[i] ^= X[i - 1];
    t = 0;
    for (Q = M; Q > 1; Q >>= 1)
        if (X[2] & Q) t ^= Q - 1;
    for (int i = 0; i < 3; i++) X[i] ^= t;
    unsigned long long h = 0;
    for (int b = bits - 1; b >= 0; b--)
        for (int i = 0; i < 3; i++) h = (h << 1) | ((X[i] >> b) & 1u);
    return h;
}

template <class T>
cudaError_t dalloc(T **p, size_t count)
{
    return cudaMalloc((void **)p, sizeof(T) * (count > 0 ? count : 1));
}

md_status fail(md_ctx *c, md_status s, const std::string &msg)
{
    if (c) c->last_error = msg;
    g_last_error = msg;
    return s;
}

void free_device(md_ctx *c)
{
    void *ptrs[] = {c->x, c->v, c->mass, c->kick, c->pos4, c->pos4_alt, c->pos_old, c->type, c->perm, c->iperm, c->f,
                    c->vir, c->epot, c->nl, c->nl_n, c->excl_orig, c->excl_s, c->cell_rank, c->cell_lin,
                    c->cell_count, c->cell_start, c->cell_fill, c->cell_work, c->key, c->src, c->tmp_d, c->tmp4,
                    c->tmp_i, c->bl_o, c->bl_on, c->al_o, c->al_on, c->bl_s, c->bl_sn, c->al_s,
                    c->al_sn, c->st, c->rec, c->lj_dev, c->bonded_par,
                    c->type_mask_dev, c->io_dev, c->reps_dev, c->repst, c->arep, c->crep,
                    c->ljr_dev, c->grid_tab, c->rep_upd, c->racc, c->p64_dev, c->rep_hist, c->snap};
    for (void *p : ptrs)
        if (p) cudaFree(p);
}

md_status check_overflow_and_sync(md_ctx *c)
{
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    md_devstate h;
    MD_CUDA_TRY(c, cudaMemcpy(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost));
    if (h.status & 2)
        return fail(c, MD_ERR_BOX,
                    "NPT: a replica's box shrank below its cell grid within one step chunk, or below "
                    "twice the list radius; create the context again from the current positions and "
                    "boxes (md_get_positions, md_get_replica_box), with a shorter cutoff or skin for the "
                    "latter");
    if (h.status != 0)
        return fail(c, MD_ERR_CUDA, "a grid barrier of the list rebuild timed out (device state invalid)");
    if (h.list_overflow > 0)
        return fail(c, MD_ERR_LIST_OVERFLOW,
                    "neighbour list overflow: " + std::to_string(h.list_overflow) + " > capacity " +
                        std::to_string(c->cap));
    return MD_OK;
}

md_status alloc_list(md_ctx *c, int cap)
{
    if (c->nl) cudaFree(c->nl);
    c->nl = nullptr;
    c->cap = cap;
    MD_CUDA_TRY(c, dalloc(&c->nl, (size_t)cap * c->pitch));
    return MD_OK;
}

/* Launch the kernels of `nsteps` steps eagerly (outside a graph): the list
 * kernels return at once unless the previous step's check asked for a build. */
void enqueue_steps(md_ctx *c, int nsteps, int energy_first)
{
    md_kparams kp = md_make_kparams(c);
    for (int k = 0; k < nsteps; k++) {
        int energy = (energy_first && k == 0) ? 1 : 0;
        if (c->integrator == MD_LEAPFROG) {
            launch_rebuild(c, kp, false, false);
            if (!energy && md_can_fuse(c)) {
                launch_pair_leapfrog(c, kp, 0, 0);
            } else {
                launch_forces(c, kp, energy != 0, MD_TERM_ALL);
                launch_leapfrog(c, kp, energy, 0, 0);
            }
        } else {
            launch_vv_first(c, kp, 0, 0);
            launch_rebuild(c, kp, false, false);
            launch_forces(c, kp, energy != 0, MD_TERM_ALL);
            launch_vv_second(c, kp, energy);
        }
    }
}

/* Inside a capture on c->stream: a conditional (if) node whose body is the
 * list rebuild, captured through c->stream2. */
md_status capture_rebuild_node(md_ctx *c, const md_kparams &kp, cudaGraphConditionalHandle h)
{
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    MD_CUDA_TRY(c, cudaStreamGetCaptureInfo(c->stream, &cs, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeIf;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    MD_CUDA_TRY(c, cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
    MD_CUDA_TRY(c, cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1,
                                                       cudaStreamSetCaptureDependencies));
    cudaGraph_t body = p.conditional.phGraph_out[0];
    MD_CUDA_TRY(c, cudaStreamBeginCaptureToGraph(c->stream2, body, nullptr, nullptr, 0,
                                                 cudaStreamCaptureModeThreadLocal));
    cudaStream_t keep = c->stream;
    c->stream = c->stream2;
    launch_rebuild(c, kp, true, false);
    c->stream = keep;
    cudaGraph_t out = nullptr;
    MD_CUDA_TRY(c, cudaStreamEndCapture(c->stream2, &out));
    return MD_OK;
}

/* A graph of `nsteps` steps.  Each step's rebuild is a conditional node set
 * by the kernel that performed the displacement check, so a step without a
 * rebuild costs only its force and integration kernels. */
md_status capture_graph(md_ctx *c, int nsteps, int energy_first)
{
    if (c->gexec) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    md_kparams kp = md_make_kparams(c);
    cudaGraph_t g = nullptr;
    MD_CUDA_TRY(c, cudaGraphCreate(&g, 0));
    /* a batch keeps the conditional node (its passes gate on per-replica flags) */
    const bool inl = c->rebuild_inline && !c->batch;
    std::vector<cudaGraphConditionalHandle> h(nsteps, 0);
    for (int k = 0; k < (inl ? 0 : nsteps); k++) {
        cudaError_t e = cudaGraphConditionalHandleCreate(&h[k], g, 0, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            return fail(c, MD_ERR_CUDA, std::string("conditional handle: ") + cudaGetErrorString(e));
        }
    }
    cudaError_t e = cudaStreamBeginCaptureToGraph(c->stream, g, nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return fail(c, MD_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    }
    md_status s = MD_OK;
    const float4 *start_pos4 = c->pos4;
    if (c->integrator == MD_LEAPFROG && !inl) launch_set_condition(c, (unsigned long long)h[0]);
    int fused = 0;
    for (int k = 0; k < nsteps && s == MD_OK; k++) {
        int energy = (energy_first && k == 0) ? 1 : 0;
        if (c->integrator == MD_LEAPFROG) {
            if (inl) launch_rebuild(c, kp, false, false, true);
            else s = capture_rebuild_node(c, kp, h[k]);
            if (s != MD_OK) break;
            int next = k + 1 < nsteps;
            /* with inline passes no kernel sets a condition */
            unsigned long long hn = (next && !inl) ? (unsigned long long)h[k + 1] : 0ull;
            /* an even number of fused steps brings the position buffers back
             * to where the graph started */
            bool fuse = !energy && md_can_fuse(c) && (next || (fused & 1));
            const int has = next && !inl;
            if (fuse) {
                launch_pair_leapfrog(c, kp, hn, has);
                fused++;
            } else {
                launch_forces(c, kp, energy != 0, MD_TERM_ALL);
                launch_leapfrog(c, kp, energy, hn, has);
            }
        } else {
            launch_vv_first(c, kp, inl ? 0ull : (unsigned long long)h[k], inl ? 0 : 1);
            if (inl) launch_rebuild(c, kp, false, false, true);
            else s = capture_rebuild_node(c, kp, h[k]);
            if (s != MD_OK) break;
            launch_forces(c, kp, energy != 0, MD_TERM_ALL);
            launch_vv_second(c, kp, energy);
        }
    }
    cudaGraph_t out = nullptr;
    e = cudaStreamEndCapture(c->stream, &out);
    if (c->pos4 != start_pos4) {   /* capture failed part way: restore the buffers */
        float4 *t = c->pos4;
        c->pos4 = c->pos4_alt;
        c->pos4_alt = t;
    }
    if (s != MD_OK) {
        cudaGraphDestroy(g);
        return s;
    }
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return fail(c, MD_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    }
    e = cudaGraphInstantiate(&c->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(c, MD_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    c->gsteps = nsteps;
    c->genergy = energy_first;
    c->gpos4 = c->pos4;
    return MD_OK;
}

md_status initial_build(md_ctx *c)
{
    md_kparams kp = md_make_kparams(c);
    launch_rebuild(c, kp, true, true);
    md_status s = check_overflow_and_sync(c);
    if (s == MD_ERR_LIST_OVERFLOW) {
        md_devstate h;
        MD_CUDA_TRY(c, cudaMemcpy(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost));
        int cap = ((h.list_overflow * 5 / 4 + 16) + 31) / 32 * 32;
        md_status a = alloc_list(c, cap);
        if (a != MD_OK) return a;
        int zero = 0;
        MD_CUDA_TRY(c, cudaMemcpy(&c->st->list_overflow, &zero, sizeof(int), cudaMemcpyHostToDevice));
        kp = md_make_kparams(c);
        launch_rebuild(c, kp, true, true);
        s = check_overflow_and_sync(c);
    }
    return s;
}

/* Forces (and KE/T) of the current state, so VV can start and records exist. */
md_status refresh_state(md_ctx *c)
{
    md_kparams kp = md_make_kparams(c);
    launch_forces(c, kp, true, MD_TERM_ALL);
    launch_thermo_from_state(c, kp, 1);
    return check_overflow_and_sync(c);
}

/* Cells of side >= rl/2 along each axis, the stencil (cells within rl; -1 =
 * every cell when the stencil would wrap onto itself) and the cells' ranks
 * along a 3-D Hilbert curve. */
struct cell_grid {
    int ncell[3], stencil[3], ncells;
    float binlen[3];
    std::vector<int> rank;   /* linear cell index -> Hilbert rank */
    std::vector<int> lin;    /* Hilbert rank -> linear cell index */
};

void make_cell_grid(const float box[3], float rl, cell_grid &g)
{
    int bits = 1;
    for (int k = 0; k < 3; k++) {
        int nc = (int)floorf(box[k] / (0.5f * rl * 1.0001f));
        nc = std::max(1, std::min(nc, 1024));
        g.ncell[k] = nc;
        g.binlen[k] = box[k] / (float)nc;
        int sten = (int)ceilf(rl / g.binlen[k]);
        g.stencil[k] = (2 * sten + 1 >= nc) ? -1 : sten;
        while ((1 << bits) < nc) bits++;
    }
    g.ncells = g.ncell[0] * g.ncell[1] * g.ncell[2];
    std::vector<std::pair<unsigned long long, int>> hk(g.ncells);
    for (int z = 0; z < g.ncell[2]; z++)
        for (int y = 0; y < g.ncell[1]; y++)
            for (int x = 0; x < g.ncell[0]; x++) {
                int lin = x + g.ncell[0] * (y + g.ncell[1] * z);
                hk[lin] = std::make_pair(hilbert3(x, y, z, bits), lin);
            }
    std::sort(hk.begin(), hk.end());
    g.rank.assign(g.ncells, 0);
    g.lin.assign(g.ncells, 0);
    for (int r = 0; r < g.ncells; r++) {
        g.rank[hk[r].second] = r;
        g.lin[r] = hk[r].second;
    }
}

/* Host staging of everything uploaded at creation, in the initial (original)
 * atom order, pitch-sized. */
struct host_stage {
    std::vector<double> x, v, m, mi;   /* mi: the kick factor dt/m * 2^-32 */
    std::vector<float4> p4;
    std::vector<int> type;
    std::vector<uint4> excl;
    std::vector<int> cell_rank, cell_lin;
    std::vector<int2> blo;      /* bonded lists (empty without bonds or angles) */
    std::vector<int> blon;
    std::vector<int4> alo;
    std::vector<int> alon;
    std::vector<float> ljh, bp;
    /* batches */
    std::vector<int> arep, crep;
    std::vector<float2> ljr;
    std::vector<int2> grid;
    std::vector<md_repstate> repst;

    void init(size_t P)
    {
        x.assign(3 * P, 0.0);
        v.assign(3 * P, 0.0);
        m.assign(P, 1.0);
        mi.assign(P, 1.0);
        p4.assign(P, make_float4(0, 0, 0, 0));
        type.assign(P, 0);
        excl.assign(P, make_uint4(MD_EXCL_NONE, MD_EXCL_NONE, MD_EXCL_NONE, MD_EXCL_NONE));
        ljh.assign(2 * MD_MAXTYPE * MD_MAXTYPE, 0.0f);
        bp.assign(4 * MD_MAXTYPE, 0.0f);
    }
};

/* Streams, device memory, upload, first list build and force evaluation of
 * a context whose host fields are set; frees everything on failure. */
md_status setup_device(md_ctx *c, void *stream, host_stage &h, md_ctx **out)
{
    if (stream) {
        c->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
            md_status s = fail(c, MD_ERR_CUDA, "stream creation failed");
            delete c;
            return s;
        }
        c->own_stream = true;
    }
    if (cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess) {
        md_status s = fail(c, MD_ERR_CUDA, "stream creation failed");
        if (c->own_stream) cudaStreamDestroy(c->stream);
        delete c;
        return s;
    }
    cudaGetDevice(&c->device);
    const size_t P = c->pitch;
    const int n = c->n;
    const bool batch = c->batch;
    cudaError_t e = cudaSuccess;
#define MD_ALLOC(ptr, cnt) if (e == cudaSuccess) e = dalloc(&(ptr), (cnt))
    MD_ALLOC(c->x, 3 * P); MD_ALLOC(c->v, 3 * P); MD_ALLOC(c->mass, P); MD_ALLOC(c->kick, P);
    MD_ALLOC(c->pos4, P); MD_ALLOC(c->pos4_alt, P); MD_ALLOC(c->pos_old, P);
    MD_ALLOC(c->type, P); MD_ALLOC(c->perm, P); MD_ALLOC(c->iperm, P);
    MD_ALLOC(c->f, 3 * P); MD_ALLOC(c->vir, P); MD_ALLOC(c->epot, P);
    MD_ALLOC(c->nl_n, P);
    MD_ALLOC(c->excl_orig, P); MD_ALLOC(c->excl_s, P);
    MD_ALLOC(c->cell_rank, c->ncells); MD_ALLOC(c->cell_lin, c->ncells); MD_ALLOC(c->cell_count, c->ncells);
    MD_ALLOC(c->cell_start, c->ncells + 1); MD_ALLOC(c->cell_fill, c->ncells); MD_ALLOC(c->cell_work, c->ncells);
    MD_ALLOC(c->key, P); MD_ALLOC(c->src, P);
    MD_ALLOC(c->tmp_d, 8 * P); MD_ALLOC(c->tmp4, P); MD_ALLOC(c->tmp_i, 3 * P);
    MD_ALLOC(c->bl_o, 4 * P); MD_ALLOC(c->bl_on, P); MD_ALLOC(c->al_o, 4 * P); MD_ALLOC(c->al_on, P);
    MD_ALLOC(c->bl_s, 4 * P); MD_ALLOC(c->bl_sn, P); MD_ALLOC(c->al_s, 4 * P); MD_ALLOC(c->al_sn, P);
    MD_ALLOC(c->st, 1);
    c->rec_cap = 4096;
    MD_ALLOC(c->rec, c->rec_cap);
    MD_ALLOC(c->lj_dev, 2 * MD_MAXTYPE * MD_MAXTYPE);
    MD_ALLOC(c->bonded_par, 4 * MD_MAXTYPE);
    MD_ALLOC(c->type_mask_dev, MD_MAXTYPE);
    MD_ALLOC(c->io_dev, 4 * P);
    if (batch) {
        MD_ALLOC(c->reps_dev, c->nrep); MD_ALLOC(c->repst, c->nrep);
        MD_ALLOC(c->arep, P); MD_ALLOC(c->crep, c->ncells);
        MD_ALLOC(c->rep_upd, c->nrep); MD_ALLOC(c->racc, 3 * (size_t)c->nrep);
        MD_ALLOC(c->ljr_dev, (size_t)MD_MAXTYPE * MD_MAXTYPE * c->nrep);
        MD_ALLOC(c->grid_tab, h.grid.size());
        MD_ALLOC(c->rep_hist, (size_t)c->rec_cap * 3 * c->nrep);
    }
#undef MD_ALLOC
    if (e != cudaSuccess) {
        md_status s = fail(c, MD_ERR_CUDA, std::string("device allocation: ") + cudaGetErrorString(e));
        free_device(c);
        if (c->own_stream) cudaStreamDestroy(c->stream);
        cudaStreamDestroy(c->stream2);
        delete c;
        return s;
    }
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);
    std::vector<int> hperm(P);
    for (size_t i = 0; i < P; i++) hperm[i] = (int)i;
    md_devstate hs;
    memset(&hs, 0, sizeof(hs));
    hs.temper = c->temper_0;   /* integrator.cu:77 */
    hs.vscale = 1.0;
    hs.lambda = 1.0;
    hs.lam_next = 1.0;     /* T_prev = T0 on the first step (integrator.cu:77) */
    hs.kick_scale = 1.0;
    std::vector<int> zeros(c->ncells, 0);
    auto up = [&](void *dst, const void *srcp, size_t bytes) {
        if (e == cudaSuccess && bytes > 0) e = cudaMemcpy(dst, srcp, bytes, cudaMemcpyHostToDevice);
    };
    up(c->x, h.x.data(), sizeof(double) * 3 * P);
    up(c->v, h.v.data(), sizeof(double) * 3 * P);
    up(c->mass, h.m.data(), sizeof(double) * P);
    up(c->kick, h.mi.data(), sizeof(double) * P);
    up(c->pos4, h.p4.data(), sizeof(float4) * P);
    up(c->type, h.type.data(), sizeof(int) * P);
    up(c->perm, hperm.data(), sizeof(int) * P);
    up(c->iperm, hperm.data(), sizeof(int) * P);
    up(c->excl_orig, h.excl.data(), sizeof(uint4) * P);
    /* without bonds there are no exclusions to remap: the sorted copy, all
     * empty, is set once */
    if (!c->has_bonds) up(c->excl_s, h.excl.data(), sizeof(uint4) * P);
    up(c->cell_rank, h.cell_rank.data(), sizeof(int) * c->ncells);
    up(c->cell_lin, h.cell_lin.data(), sizeof(int) * c->ncells);
    up(c->cell_count, zeros.data(), sizeof(int) * c->ncells);
    up(c->cell_fill, zeros.data(), sizeof(int) * c->ncells);
    if (!h.blo.empty()) {
        up(c->bl_o, h.blo.data(), sizeof(int2) * 4 * n);
        up(c->bl_on, h.blon.data(), sizeof(int) * n);
        up(c->al_o, h.alo.data(), sizeof(int4) * 4 * n);
        up(c->al_on, h.alon.data(), sizeof(int) * n);
    } else {
        if (e == cudaSuccess) e = cudaMemset(c->bl_on, 0, sizeof(int) * P);
        if (e == cudaSuccess) e = cudaMemset(c->al_on, 0, sizeof(int) * P);
    }
    up(c->lj_dev, h.ljh.data(), sizeof(float) * h.ljh.size());
    up(c->bonded_par, h.bp.data(), sizeof(float) * h.bp.size());
    up(c->type_mask_dev, c->type_excl_mask, sizeof(unsigned) * MD_MAXTYPE);
    up(c->st, &hs, sizeof(hs));
    if (batch) {
        up(c->reps_dev, c->reps.data(), sizeof(md_rep) * c->nrep);
        up(c->repst, h.repst.data(), sizeof(md_repstate) * c->nrep);
        up(c->arep, h.arep.data(), sizeof(int) * P);
        up(c->crep, h.crep.data(), sizeof(int) * c->ncells);
        up(c->ljr_dev, h.ljr.data(), sizeof(float2) * h.ljr.size());
        up(c->grid_tab, h.grid.data(), sizeof(int2) * h.grid.size());
        if (e == cudaSuccess) e = cudaMemset(c->rep_upd, 0, sizeof(int) * c->nrep);
        if (e == cudaSuccess) e = cudaMemset(c->racc, 0, sizeof(unsigned long long) * 3 * c->nrep);
    }
    if (e == cudaSuccess) e = cudaMemset(c->f, 0, sizeof(long long) * 3 * P);
    if (e == cudaSuccess) e = cudaMemset(c->vir, 0, sizeof(float) * P);
    if (e == cudaSuccess) e = cudaMemset(c->epot, 0, sizeof(float) * P);
    if (e == cudaSuccess) e = cudaMemset(c->bl_sn, 0, sizeof(int) * P);
    if (e == cudaSuccess) e = cudaMemset(c->al_sn, 0, sizeof(int) * P);
    if (e == cudaSuccess) e = cudaMemset(c->nl_n, 0, sizeof(int) * P);
    if (e != cudaSuccess) {
        md_status s = fail(c, MD_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
        md_destroy(c);
        return s;
    }
    md_status s = alloc_list(c, (c->nmaxlist + 31) / 32 * 32);
    if (s == MD_OK) s = initial_build(c);
    if (s == MD_OK) s = refresh_state(c);
    if (s != MD_OK) {
        g_last_error = c->last_error;
        md_destroy(c);
        return s;
    }
    *out = c;
    return MD_OK;
}

}  // namespace

void md_set_global_error(const std::string &msg) { g_last_error = msg; }

int md_cell_shift(const int stencil[3], const float binlen[3], const float box[3])
{
    for (int d = 0; d < 3; d++)
        if (stencil[d] < 0 || (stencil[d] + 1) * (double)binlen[d] >= 0.49 * (double)box[d]) return 0;
    return 1;
}

int md_ndf(const md_ctx *c)
{
    if (c->batch) {
        long long s = 0;
        for (const md_rep &r : c->reps) s += r.ndf;
        return (int)s;
    }
    return std::max(1, 3 * c->n - 3);
}

md_kparams md_make_kparams(const md_ctx *c)
{
    md_kparams kp;
    memset(&kp, 0, sizeof(kp));
    kp.n = c->n;
    kp.pitch = c->pitch;
    kp.cap = c->cap;
    kp.ntype = c->ntype;
    for (int d = 0; d < 3; d++) {
        kp.box[d] = c->box[d];
        kp.boxi[d] = c->boxi[d];
        kp.boxd[d] = (double)c->box[d];
        kp.box2i[d] = 2.0 / (double)c->box[d];
        kp.wlim[d] = 0.4999f * c->box[d];
        kp.ncell[d] = c->ncell[d];
        kp.binlen[d] = c->binlen[d];
        kp.stencil[d] = c->stencil[d];
    }
    /* the image shift by stencil cell holds when positions lie in the box */
    kp.cell_shift = c->centered && md_cell_shift(c->stencil, c->binlen, c->box);
    kp.rcutsq = c->rcutsq;
    kp.reacf = c->reacf;
    kp.rskinsq = c->rskinsq;
    kp.rmaxdif = c->rmaxdif;
    kp.palfa = c->wc[0];
    kp.spiialfa = c->wc[1];
    kp.alfasq = c->wc[2];
    kp.wolf = c->wc[3];
    kp.lkspace = c->lkspace;
    kp.dt = c->dt;
    kp.centered = c->centered;
    return kp;
}

/* Whether every position of n atoms (3 per atom) lies in [-L/2, L/2] on
 * each axis, as FP32.  Once it holds, the integrators' wrap keeps it (a
 * step moves an atom far less than L/2), so the cells may take the image
 * shift by stencil cell and the pair kernels may skip the minimum-image
 * shifts of atoms at least rc from every face. */
template <typename T>
static bool centered_range(const T *pos3, int n, const float *box)
{
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++)
            if (!(fabsf((float)pos3[3 * (size_t)i + k]) <= 0.5f * box[k])) return false;
    return true;
}

extern "C" {

const char *md_status_string(md_status s)
{
    switch (s) {
    case MD_OK: return "ok";
    case MD_ERR_ARG: return "invalid argument";
    case MD_ERR_IO: return "cannot open file";
    case MD_ERR_PARSE: return "input does not follow the .inp/.fld/.cfg grammar";
    case MD_ERR_CUDA: return "CUDA error";
    case MD_ERR_LIST_OVERFLOW: return "neighbour list overflow";
    case MD_ERR_BONDED: return "more than four bonds or angles on an atom";
    case MD_ERR_UNSUPPORTED: return "unsupported option";
    case MD_ERR_BOX: return "cutoff plus skin exceeds half the box";
    }
    return "unknown status";
}

md_status md_last_error(const md_ctx *ctx, char *buf, int len)
{
    if (!buf || len <= 0) return MD_ERR_ARG;
    const std::string &m = ctx ? ctx->last_error : g_last_error;
    snprintf(buf, (size_t)len, "%s", m.c_str());
    return MD_OK;
}

/* Exclusions with the reference's slot rule and the per-atom bonded lists
 * of c->bonds / c->angles (n atoms, indices in the context's atom space);
 * sets has_bonds / has_angles.  Errors leave c to the caller. */
md_status bonded_lists(md_ctx *c, int n, std::vector<int2> &blo, std::vector<int> &blon,
                       std::vector<int4> &alo, std::vector<int> &alon)
{
    /* exclusions with the reference's slot rule (neighborlist.cu:64-97) */
    c->excl_host.assign(4 * (size_t)n, MD_EXCL_NONE);
    for (size_t b = 0; b < c->bonds.size() / 3; b++) {
        unsigned i = (unsigned)c->bonds[3 * b + 1], j = (unsigned)c->bonds[3 * b + 2];
        if (i >= (unsigned)n || j >= (unsigned)n) {
            return fail(c, MD_ERR_ARG, "bond atom out of range");
        }
        unsigned *ei = &c->excl_host[4 * i], *ej = &c->excl_host[4 * j];
        auto empty = [](unsigned v) { return v == MD_EXCL_NONE; };
        if (empty(ei[0])) ei[0] = j;
        else if (empty(ei[1])) ei[1] = j;
        else if (empty(ei[2])) ei[2] = j;
        else if (empty(ei[3])) ei[3] = j;
        if (empty(ej[0])) ej[0] = i;
        else if (empty(ei[1])) ej[1] = i;
        else if (empty(ei[2])) ej[2] = i;
        else if (empty(ei[3])) ej[3] = i;
    }
    /* original-space bonded lists (forces.cu:118-173), at most four per atom */
    blo.assign(4 * (size_t)n, make_int2(0, 0));
    blon.assign(n, 0);
    alo.assign(4 * (size_t)n, make_int4(0, 0, 0, 0));
    alon.assign(n, 0);
    for (size_t b = 0; b < c->bonds.size() / 3; b++) {
        int t = c->bonds[3 * b], i = c->bonds[3 * b + 1], j = c->bonds[3 * b + 2];
        if (blon[i] >= 4 || blon[j] >= 4) {
            return fail(c, MD_ERR_BONDED, "more than four bonds on an atom");
        }
        blo[4 * i + blon[i]++] = make_int2(j, t);
        blo[4 * j + blon[j]++] = make_int2(i, t);
    }
    for (size_t a = 0; a < c->angles.size() / 4; a++) {
        int t = c->angles[4 * a], i = c->angles[4 * a + 1], j = c->angles[4 * a + 2],
            k = c->angles[4 * a + 3];
        if (i < 0 || j < 0 || k < 0 || i >= n || j >= n || k >= n || alon[i] >= 4 || alon[j] >= 4 ||
            alon[k] >= 4) {
            return fail(c, MD_ERR_BONDED, "more than four angles on an atom (or bad index)");
        }
        alo[4 * i + alon[i]++] = make_int4(0, j, k, t);
        alo[4 * j + alon[j]++] = make_int4(1, i, k, t);
        alo[4 * k + alon[k]++] = make_int4(0, j, i, t);
    }
    c->has_bonds = c->bonds.empty() ? 0 : 1;
    c->has_angles = c->angles.empty() ? 0 : 1;
    return MD_OK;
}

md_status md_create(const md_system_desc *d, void *stream, md_ctx **out)
{
    if (!d || !out || d->natom <= 0 || d->ntype < 1 || d->ntype > MD_MAXTYPE || !d->itype ||
        !d->charge || !d->pos || !d->type_mass || !d->lj1 || !d->lj2)
        return fail(nullptr, MD_ERR_ARG, "md_create: missing or invalid descriptor fields");
    if (d->nbonds > 0 && (!d->bonds || !d->bnd1 || !d->bnd2))
        return fail(nullptr, MD_ERR_ARG, "md_create: bonds without tables");
    if (d->nangle > 0 && (!d->angles || !d->ang1 || !d->ang2))
        return fail(nullptr, MD_ERR_ARG, "md_create: angles without tables");
    if (d->lkspace < 0 || d->lkspace > 2 || d->rcutsq <= 0 || d->skin < 0 || d->dt <= 0 ||
        d->integrator < 0 || d->integrator > 2 || d->enstype < 0 || d->enstype > 2)
        return fail(nullptr, MD_ERR_ARG, "md_create: invalid run parameters");
    /* NPT: the box becomes a per-step device quantity, which the batch kernels
     * read from their replica table; a single NPT system is a batch of one */
    if (d->enstype == 2) return md_create_batch(d, 1, stream, out);
    md_ctx *c = new (std::nothrow) md_ctx();
    if (!c) return fail(nullptr, MD_ERR_ARG, "out of host memory");
    const int n = d->natom;
    c->n = n;
    c->ntype = d->ntype;
    c->pitch = ((n + 255) / 256) * 256;
    for (int k = 0; k < 3; k++) {
        c->box[k] = d->box[k];
        c->boxi[k] = (float)(1.0 / (double)d->box[k]);   /* simulation.cu:290-292 */
    }
    c->lkspace = d->lkspace;
    c->rcutsq = d->rcutsq;
    c->reacf = d->lkspace == 0 ? d->reacf : 0.0f;
    c->alfa = d->alfa;
    c->skin = d->skin;
    c->nmaxlist = d->nmaxlist > 0 ? d->nmaxlist : 64;
    c->enstype = d->enstype;
    c->temper_0 = d->temper_0;
    c->dt = d->dt;
    c->tau_t = d->tau_t > 0 ? d->tau_t : 100.0f;
    c->integrator = d->integrator;
    if (c->lkspace > 0) wolf_consts(c->alfa, c->rcutsq, c->wc);
    if (c->lkspace != 1) c->wc[3] = 0.0f;
    c->rskinsq = (float)pow((double)(c->skin + sqrtf(c->rcutsq)), 2.0);   /* neighborlist.cu:35 */
    c->rmaxdif = c->skin * c->skin / 4.0f;                                /* neighborlist.cu:36 */
    float rl = sqrtf(c->rcutsq) + c->skin;
    for (int k = 0; k < 3; k++)
        if (2.0f * rl > c->box[k]) {
            md_status s = fail(c, MD_ERR_BOX, "cutoff + skin exceeds half the box");
            delete c;
            return s;
        }
    memset(c->lj1, 0, sizeof(c->lj1));
    memset(c->lj2, 0, sizeof(c->lj2));
    for (int k = 0; k < d->ntype * d->ntype; k++) {
        c->lj1[k] = d->lj1[k];
        c->lj2[k] = d->lj2[k];
    }
    for (int k = 0; k < MD_MAXTYPE; k++) {
        c->bnd1[k] = d->bnd1 && d->nbonds > 0 ? d->bnd1[k] : 0.0f;
        c->bnd2[k] = d->bnd2 && d->nbonds > 0 ? d->bnd2[k] : 0.0f;
        c->ang1[k] = d->ang1 && d->nangle > 0 ? d->ang1[k] : 0.0f;
        c->ang2[k] = d->ang2 && d->nangle > 0 ? d->ang2[k] : 0.0f;
        c->type_mass[k] = k < d->ntype ? d->type_mass[k] : 0.0f;
    }
    c->itype.assign(d->itype, d->itype + n);
    c->charge.assign(d->charge, d->charge + n);
    for (int i = 0; i < n; i++)
        if (c->itype[i] < 0 || c->itype[i] >= d->ntype) {
            md_status s = fail(c, MD_ERR_ARG, "atom type out of range");
            delete c;
            return s;
        }
    if (d->nbonds > 0) c->bonds.assign(d->bonds, d->bonds + 3 * (size_t)d->nbonds);
    if (d->nangle > 0) c->angles.assign(d->angles, d->angles + 4 * (size_t)d->nangle);

    std::vector<int2> blo;
    std::vector<int> blon;
    std::vector<int4> alo;
    std::vector<int> alon;
    {
        md_status bs = bonded_lists(c, n, blo, blon, alo, alon);
        if (bs != MD_OK) {
            delete c;
            return bs;
        }
    }
    c->has_bonds = c->bonds.empty() ? 0 : 1;
    c->has_angles = c->angles.empty() ? 0 : 1;

    /* cells of side >= rl/2 and their Hilbert ranks */
    cell_grid g;
    make_cell_grid(c->box, rl, g);
    for (int k = 0; k < 3; k++) {
        c->ncell[k] = g.ncell[k];
        c->binlen[k] = g.binlen[k];
        c->stencil[k] = g.stencil[k];
    }
    c->ncells = g.ncells;

    /* host staging in sorted order = original order before the first build */
    host_stage h;
    h.init(c->pitch);
    const size_t P = c->pitch;
    c->centered = centered_range(d->pos, n, c->box) ? 1 : 0;
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < 3; k++) {
            h.x[k * P + i] = d->pos[3 * i + k];
            h.v[k * P + i] = d->vel ? d->vel[3 * i + k] : 0.0;
        }
        h.m[i] = c->type_mass[c->itype[i]];
        h.mi[i] = ((double)c->dt * (1.0 / h.m[i])) * FX_INV;
        h.p4[i] = make_float4(d->pos[3 * i], d->pos[3 * i + 1], d->pos[3 * i + 2], c->charge[i]);
        h.type[i] = c->itype[i];
        h.excl[i] = make_uint4(c->excl_host[4 * i], c->excl_host[4 * i + 1], c->excl_host[4 * i + 2],
                               c->excl_host[4 * i + 3]);
    }
    h.cell_rank = std::move(g.rank);
    h.cell_lin = std::move(g.lin);
    h.blo = std::move(blo);
    h.blon = std::move(blon);
    h.alo = std::move(alo);
    h.alon = std::move(alon);
    for (int a = 0; a < c->ntype; a++)
        for (int b = 0; b < c->ntype; b++) {
            h.ljh[2 * (a * MD_MAXTYPE + b)] = c->lj1[a * c->ntype + b];
            h.ljh[2 * (a * MD_MAXTYPE + b) + 1] = c->lj2[a * c->ntype + b];
        }
    for (int k = 0; k < MD_MAXTYPE; k++) {
        h.bp[k] = c->bnd1[k]; h.bp[MD_MAXTYPE + k] = c->bnd2[k];
        h.bp[2 * MD_MAXTYPE + k] = c->ang1[k]; h.bp[3 * MD_MAXTYPE + k] = c->ang2[k];
    }
    return setup_device(c, stream, h, out);
}

/* bar per kJ/mol/A^3 (1 kJ/mol/A^3 = 1.66053907e9 Pa) */
constexpr double MD_BAR = 16605.3907;

/* The Berendsen barostat's constants of every replica of an NPT batch from
 * c->baro (target pressure in bar, tau_p in fs, compressibility in 1/bar):
 * mu = 1 - beta dt / (3 tau_p) (P0 - P), pressures in kJ/mol/A^3. */
static void apply_barostat(md_ctx *c)
{
    for (md_rep &R : c->reps) {
        if (!R.npt) continue;
        R.p0 = c->baro[0] / MD_BAR;
        R.mu_k = c->baro[2] * MD_BAR * (double)c->dt / (3.0 * c->baro[1]);
    }
}

md_status md_create_batch(const md_system_desc *descs, int nrep, void *stream, md_ctx **out)
{
    if (!descs || !out || nrep < 1) return fail(nullptr, MD_ERR_ARG, "md_create_batch: null argument");

    const md_system_desc &d0 = descs[0];
    long long ntot = 0;
    int ntype = 1, nmax = 0;
    for (int r = 0; r < nrep; r++) {
        const md_system_desc *d = descs + r;
        std::string at = " (replica " + std::to_string(r) + ")";
        if (d->natom <= 0 || d->ntype < 1 || d->ntype > MD_MAXTYPE || !d->itype || !d->charge ||
            !d->pos || !d->type_mass || !d->lj1 || !d->lj2)
            return fail(nullptr, MD_ERR_ARG, "md_create_batch: missing or invalid descriptor fields" + at);
        if ((d->nbonds > 0 && (!d->bonds || !d->bnd1 || !d->bnd2)) ||
            (d->nangle > 0 && (!d->angles || !d->ang1 || !d->ang2)))
            return fail(nullptr, MD_ERR_ARG, "md_create_batch: bonded terms without tables" + at);
        /* one bonded parameter table for the batch: the bonded kernels read
         * one set (every replica that has bonds or angles must carry it) */
        for (int q = 0; q < r; q++) {
            const md_system_desc *e = descs + q;
            if ((d->nbonds > 0 && e->nbonds > 0 &&
                 (memcmp(d->bnd1, e->bnd1, sizeof(float) * MD_MAXTYPE) ||
                  memcmp(d->bnd2, e->bnd2, sizeof(float) * MD_MAXTYPE))) ||
                (d->nangle > 0 && e->nangle > 0 &&
                 (memcmp(d->ang1, e->ang1, sizeof(float) * MD_MAXTYPE) ||
                  memcmp(d->ang2, e->ang2, sizeof(float) * MD_MAXTYPE))))
                return fail(nullptr, MD_ERR_ARG,
                            "md_create_batch: replicas with different bonded parameters" + at);
        }
        if (d->lkspace < 0 || d->lkspace > 2 || d->rcutsq <= 0 || d->skin < 0 || d->dt <= 0 ||
            d->integrator < 0 || d->integrator > 2 || d->enstype < 0 || d->enstype > 2)
            return fail(nullptr, MD_ERR_ARG, "md_create_batch: invalid run parameters" + at);
        if (d->enstype == 2 && d->integrator != MD_LEAPFROG)
            return fail(nullptr, MD_ERR_UNSUPPORTED,
                        "md_create_batch: NPT runs the Berendsen leapfrog (npt_leapfrog_ber.cu)" + at);
        if (d->lkspace != d0.lkspace || d->integrator != d0.integrator || d->enstype != d0.enstype ||
            d->dt != d0.dt || d->tau_t != d0.tau_t)
            return fail(nullptr, MD_ERR_ARG,
                        "md_create_batch: replicas must share lkspace, integrator, ensemble, dt and tau_t" + at);
        for (int i = 0; i < d->natom; i++)
            if (d->itype[i] < 0 || d->itype[i] >= d->ntype)
                return fail(nullptr, MD_ERR_ARG, "md_create_batch: atom type out of range" + at);
        float rl = sqrtf(d->rcutsq) + d->skin;
        for (int k = 0; k < 3; k++)
            if (2.0f * rl > d->box[k])
                return fail(nullptr, MD_ERR_BOX, "md_create_batch: cutoff + skin exceeds half the box" + at);
        ntot += d->natom;
        ntype = std::max(ntype, d->ntype);
        nmax = std::max(nmax, d->nmaxlist > 0 ? d->nmaxlist : 64);
    }
    if (ntot >= (long long)MD_INDEX_MASK)
        return fail(nullptr, MD_ERR_ARG, "md_create_batch: too many atoms");
    md_ctx *c = new (std::nothrow) md_ctx();
    if (!c) return fail(nullptr, MD_ERR_ARG, "out of host memory");
    const int n = (int)ntot;
    c->batch = 1;
    c->nrep = nrep;
    c->n = n;
    c->ntype = ntype;
    c->pitch = ((n + 255) / 256) * 256;
    for (int k = 0; k < 3; k++) {
        c->box[k] = d0.box[k];
        c->boxi[k] = (float)(1.0 / (double)d0.box[k]);
    }
    c->lkspace = d0.lkspace;
    c->rcutsq = d0.rcutsq;
    c->reacf = d0.lkspace == 0 ? d0.reacf : 0.0f;
    c->alfa = d0.alfa;
    c->skin = d0.skin;
    c->nmaxlist = nmax;
    c->enstype = d0.enstype;
    c->temper_0 = d0.temper_0;
    c->dt = d0.dt;
    c->tau_t = d0.tau_t > 0 ? d0.tau_t : 100.0f;
    c->integrator = d0.integrator;
    if (c->lkspace > 0) wolf_consts(c->alfa, c->rcutsq, c->wc);
    if (c->lkspace != 1) c->wc[3] = 0.0f;
    c->rskinsq = (float)pow((double)(c->skin + sqrtf(c->rcutsq)), 2.0);
    c->rmaxdif = c->skin * c->skin / 4.0f;
    memset(c->lj1, 0, sizeof(c->lj1));
    memset(c->lj2, 0, sizeof(c->lj2));
    memset(c->bnd1, 0, sizeof(c->bnd1));
    memset(c->bnd2, 0, sizeof(c->bnd2));
    memset(c->ang1, 0, sizeof(c->ang1));
    memset(c->ang2, 0, sizeof(c->ang2));
    memset(c->type_mass, 0, sizeof(c->type_mass));
    c->list_tpa = 0;   /* batches build their lists one warp per cell */
    c->centered = 1;   /* cleared below by any replica with a position outside its box */
    /* bonds and angles of every replica in batch atom indices */
    {
        long long a0 = 0;
        for (int r = 0; r < nrep; r++) {
            const md_system_desc *d = descs + r;
            for (int k = 0; k < MD_MAXTYPE; k++) {
                if (d->nbonds > 0) {
                    c->bnd1[k] = d->bnd1[k];
                    c->bnd2[k] = d->bnd2[k];
                }
                if (d->nangle > 0) {
                    c->ang1[k] = d->ang1[k];
                    c->ang2[k] = d->ang2[k];
                }
            }
            for (int b = 0; b < d->nbonds; b++) {
                const int *e = d->bonds + 3 * (size_t)b;
                if (e[1] < 0 || e[2] < 0 || e[1] >= d->natom || e[2] >= d->natom) {
                    md_status s = fail(c, MD_ERR_ARG, "md_create_batch: bond atom out of range");
                    delete c;
                    return s;
                }
                c->bonds.push_back(e[0]);
                c->bonds.push_back((int)(a0 + e[1]));
                c->bonds.push_back((int)(a0 + e[2]));
            }
            for (int b = 0; b < d->nangle; b++) {
                const int *e = d->angles + 4 * (size_t)b;
                if (e[1] < 0 || e[2] < 0 || e[3] < 0 || e[1] >= d->natom || e[2] >= d->natom ||
                    e[3] >= d->natom) {
                    md_status s = fail(c, MD_ERR_ARG, "md_create_batch: angle atom out of range");
                    delete c;
                    return s;
                }
                c->angles.push_back(e[0]);
                for (int q = 1; q < 4; q++) c->angles.push_back((int)(a0 + e[q]));
            }
            a0 += d->natom;
        }
    }
    std::vector<int2> blo;
    std::vector<int> blon;
    std::vector<int4> alo;
    std::vector<int> alon;
    {
        md_status bs = bonded_lists(c, n, blo, blon, alo, alon);
        if (bs != MD_OK) {
            delete c;
            return bs;
        }
    }

    host_stage h;
    const size_t P = c->pitch;
    h.init(P);
    h.arep.assign(P, nrep - 1);
    h.ljr.assign((size_t)MD_MAXTYPE * MD_MAXTYPE * nrep, make_float2(0.0f, 0.0f));
    h.repst.resize(nrep);
    c->reps.resize(nrep);
    c->rep_natom.resize(nrep);
    c->itype.resize(n);
    c->charge.resize(n);
    int atom0 = 0, cell0 = 0;
    const double tau = c->tau_t;
    for (int r = 0; r < nrep; r++) {
        const md_system_desc *d = descs + r;
        md_rep &R = c->reps[r];
        memset(&R, 0, sizeof(R));
        for (int k = 0; k < 3; k++) {
            R.box[k] = d->box[k];
            R.boxi[k] = (float)(1.0 / (double)d->box[k]);   /* simulation.cu:290-292 */
            R.boxd[k] = (double)d->box[k];
            R.box2i[k] = 2.0 / (double)d->box[k];
            R.wlim[k] = 0.4999f * d->box[k];
        }
        R.rcutsq = d->rcutsq;
        R.reacf = d->lkspace == 0 ? d->reacf : 0.0f;
        c->rep_alfa.push_back(d->alfa);
        float wc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (d->lkspace > 0) wolf_consts(d->alfa, d->rcutsq, wc);
        R.palfa = wc[0];
        R.spiialfa = wc[1];
        R.alfasq = wc[2];
        R.wolf = d->lkspace == 1 ? wc[3] : 0.0f;
        R.rskinsq = (float)pow((double)(d->skin + sqrtf(d->rcutsq)), 2.0);   /* neighborlist.cu:35 */
        R.rmaxdif = d->skin * d->skin / 4.0f;                                 /* neighborlist.cu:36 */
        md_shift_consts(d->lkspace, d->rcutsq, d->alfa, R.reacf, &R.ucc, &R.rc6i, &R.rcinv);
        cell_grid g;
        /* NPT: cells 3% longer than half the list radius, so the box may
         * shrink that far before the stencil of +-2 cells stops covering it */
        const float rl = sqrtf(d->rcutsq) + d->skin;
        make_cell_grid(d->box, d->enstype == 2 ? rl * 1.03f : rl, g);
        R.rl_half = 0.5f * rl;
        R.npt = d->enstype == 2 ? 1 : 0;
        R.mu_max = 1e-4;
        for (int k = 0; k < 3; k++) {
            R.ncell[k] = g.ncell[k];
            R.stencil[k] = g.stencil[k];
            R.binlen[k] = g.binlen[k];
        }
        R.cell_shift = md_cell_shift(R.stencil, R.binlen, R.box);
        int nst = 1;   /* the warp-per-cell builder holds up to 128 stencil cells */
        for (int k = 0; k < 3; k++) nst *= R.stencil[k] < 0 ? R.ncell[k] : 2 * R.stencil[k] + 1;
        if (nst > 128) {
            md_status s = fail(c, MD_ERR_UNSUPPORTED, "md_create_batch: stencil too large");
            delete c;
            return s;
        }
        R.cell0 = cell0;
        R.ncells = g.ncells;
        R.atom0 = atom0;
        R.natom = d->natom;
        R.ndf = std::max(1, 3 * d->natom - 3);
        R.t0 = d->temper_0;
        R.q_nh = R.ndf * 8.314e-3 * R.t0 * tau * tau;
        if (R.q_nh <= 0) R.q_nh = 1.0;
        R.inv_ndfr = 1.0 / (R.ndf * 8.314e-3);
        R.inv_q = 1.0 / R.q_nh;
        c->rep_natom[r] = d->natom;
        /* cells: global rank = cell0 + Hilbert rank inside the replica */
        for (int k = 0; k < g.ncells; k++) {
            h.cell_rank.push_back(cell0 + g.rank[k]);
            h.cell_lin.push_back(g.lin[k]);
            h.crep.push_back(r);
        }
        for (int a = 0; a < d->ntype; a++)
            for (int b = 0; b < d->ntype; b++)
                h.ljr[(size_t)r * MD_MAXTYPE * MD_MAXTYPE + a * MD_MAXTYPE + b] =
                    make_float2(d->lj1[a * d->ntype + b], d->lj2[a * d->ntype + b]);
        if (!centered_range(d->pos, d->natom, d->box)) c->centered = 0;
        for (int i = 0; i < d->natom; i++) {
            int gi = atom0 + i;
            for (int k = 0; k < 3; k++) {
                h.x[k * P + gi] = d->pos[3 * i + k];
                h.v[k * P + gi] = d->vel ? d->vel[3 * i + k] : 0.0;
            }
            h.m[gi] = d->type_mass[d->itype[i]];
            h.mi[gi] = ((double)d->dt * (1.0 / h.m[gi])) * FX_INV;
            h.p4[gi] = make_float4(d->pos[3 * i], d->pos[3 * i + 1], d->pos[3 * i + 2], d->charge[i]);
            h.type[gi] = d->itype[i];
            h.arep[gi] = r;
            c->itype[gi] = d->itype[i];
            c->charge[gi] = d->charge[i];
        }
        md_repstate &S = h.repst[r];
        memset(&S, 0, sizeof(S));
        S.temper = R.t0;
        S.vscale = S.lambda = S.lam_next = S.kick_scale = 1.0;
        S.mu_next = S.mu_used = 1.0;
        atom0 += d->natom;
        cell0 += g.ncells;
    }
    c->ncells = cell0;
    for (int i = 0; i < n; i++)
        h.excl[i] = make_uint4(c->excl_host[4 * i], c->excl_host[4 * i + 1], c->excl_host[4 * i + 2],
                               c->excl_host[4 * i + 3]);
    if (c->has_bonds || c->has_angles) {
        h.blo = std::move(blo);
        h.blon = std::move(blon);
        h.alo = std::move(alo);
        h.alon = std::move(alon);
    }
    for (int k = 0; k < MD_MAXTYPE; k++) {
        h.bp[k] = c->bnd1[k]; h.bp[MD_MAXTYPE + k] = c->bnd2[k];
        h.bp[2 * MD_MAXTYPE + k] = c->ang1[k]; h.bp[3 * MD_MAXTYPE + k] = c->ang2[k];
    }
    for (int k = 0; k < 3; k++) {
        c->ncell[k] = c->reps[0].ncell[k];
        c->binlen[k] = c->reps[0].binlen[k];
        c->stencil[k] = c->reps[0].stencil[k];
    }
    /* replica-aligned grids of 4 .. 256 atoms per block */
    for (int k = 0; k < MD_NGRID; k++) {
        const int A = 4 << k;
        c->grid_off[k] = (int)h.grid.size();
        for (int r = 0; r < nrep; r++) {
            md_rep &R = c->reps[r];
            if (A == MD_LA) R.blk0 = (int)h.grid.size() - c->grid_off[k];
            if (A == MD_ADJ_ATOMS) R.ablk0 = (int)h.grid.size() - c->grid_off[k];
            for (int j = 0; j < R.natom; j += A) h.grid.push_back(make_int2(r, R.atom0 + j));
            if (A == MD_LA) R.nblk = (int)h.grid.size() - c->grid_off[k] - R.blk0;
            if (A == MD_ADJ_ATOMS) R.anblk = (int)h.grid.size() - c->grid_off[k] - R.ablk0;
        }
        c->grid_cnt[k] = (int)h.grid.size() - c->grid_off[k];
    }
    apply_barostat(c);
    return setup_device(c, stream, h, out);
}

md_status md_get_replica_thermo(md_ctx *c, md_thermo *out, int nrep)
{
    if (!c || !out || nrep < 1) return MD_ERR_ARG;
    if (!c->batch) return md_get_thermo(c, out);
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    md_devstate h;
    MD_CUDA_TRY(c, cudaMemcpy(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost));
    int k = std::min(nrep, c->nrep);
    std::vector<md_repstate> rs(k);
    MD_CUDA_TRY(c, cudaMemcpy(rs.data(), c->repst, sizeof(md_repstate) * k, cudaMemcpyDeviceToHost));
    int flags = 0;
    if (h.step > 0) {
        md_thermo last;
        MD_CUDA_TRY(c, cudaMemcpy(&last, c->rec + (h.step - 1) % c->rec_cap, sizeof(md_thermo),
                                  cudaMemcpyDeviceToHost));
        flags = last.flags;
    }
    const bool nh = c->integrator == MD_NH;
    for (int r = 0; r < k; r++) {
        const md_rep &R = c->reps[r];
        md_thermo &o = out[r];
        memset(&o, 0, sizeof(o));
        o.step = h.step > 0 ? h.step - 1 : 0;
        o.ke = rs[r].ke;
        o.temper = 2.0 * rs[r].ke / (R.ndf * 8.314e-3);
        o.pe = rs[r].pe;
        o.virial = rs[r].virial;
        o.conserved = rs[r].ke + rs[r].pe +
                      (nh ? 0.5 * R.q_nh * rs[r].xi * rs[r].xi + R.ndf * 8.314e-3 * R.t0 * rs[r].eta : 0.0);
        o.xi = rs[r].xi;
        o.lambda = rs[r].lambda;
        o.builds = rs[r].builds;
        o.flags = flags;
    }
    return MD_OK;
}

md_status md_create_from_files(const char *base, void *stream, md_ctx **out)
{
    if (!base || !out) return fail(nullptr, MD_ERR_ARG, "md_create_from_files: null argument");
    parsed_run r;
    memset(&r.d, 0, sizeof(r.d));
    std::string b(base);
    md_status s = parse_inp((b + ".inp").c_str(), r);
    if (s != MD_OK) return fail(nullptr, s, "reading " + b + ".inp: " + md_status_string(s));
    s = parse_fld((b + ".fld").c_str(), r);
    if (s != MD_OK) return fail(nullptr, s, "reading " + b + ".fld: " + md_status_string(s));
    s = parse_cfg((b + ".cfg").c_str(), r);
    if (s != MD_OK) return fail(nullptr, s, "reading " + b + ".cfg: " + md_status_string(s));
    for (int t : r.itype)
        if (t < 0 || t >= r.d.ntype) return fail(nullptr, MD_ERR_PARSE, "atom type out of range in .cfg");
    md_system_desc &d = r.d;
    d.itype = r.itype.data();
    d.charge = r.charge.data();
    d.pos = r.pos.data();
    d.vel = r.vel.data();
    d.type_mass = r.mass.data();
    d.lj1 = r.lj1.data();
    d.lj2 = r.lj2.data();
    d.bonds = r.bonds.data();
    d.angles = r.angles.data();
    d.bnd1 = r.bnd1.data();
    d.bnd2 = r.bnd2.data();
    d.ang1 = r.ang1.data();
    d.ang2 = r.ang2.data();
    s = md_create(&d, stream, out);
    if (s == MD_OK) {
        (*out)->timprn = r.timprn;
        (*out)->type_names = r.names;
        if (d.enstype == 2) s = md_set_barostat(*out, r.press0, r.tau_p, r.beta);
        if (s == MD_OK && d.lkspace == 2 && r.pme_spacing > 0.0f) {
            /* the fewest grid points, in multiples of 8 (at least 16),
             * that keep the spacing at most pme_spacing */
            int K[3];
            for (int k = 0; k < 3; k++)
                K[k] = std::max(16, 8 * (int)ceil((double)d.box[k] / (8.0 * r.pme_spacing)));
            s = md_set_pme(*out, K[0], K[1], K[2]);
        }
        if (s != MD_OK) {
            const std::string msg = (*out)->last_error;
            md_destroy(*out);
            *out = nullptr;
            md_set_global_error(msg);
        }
    }
    return s;
}

md_status md_destroy(md_ctx *c)
{
    if (!c) return MD_ERR_ARG;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    pme_free(c);
    free_device(c);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    delete c;
    return MD_OK;
}

static md_status gather_to_host(md_ctx *c, int what, double *dst, size_t count)
{
    md_kparams kp = md_make_kparams(c);
    launch_gather_out(c, kp, what, c->io_dev);
    MD_CUDA_TRY(c, cudaMemcpyAsync(dst, c->io_dev, sizeof(double) * count, cudaMemcpyDeviceToHost,
                                   c->stream));
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MD_OK;
}

md_status md_get_positions(md_ctx *c, double *pos3)
{
    if (!c || !pos3) return MD_ERR_ARG;
    return gather_to_host(c, 0, pos3, 3 * (size_t)c->n);
}

md_status md_get_velocities(md_ctx *c, double *vel3)
{
    if (!c || !vel3) return MD_ERR_ARG;
    return gather_to_host(c, 1, vel3, 3 * (size_t)c->n);
}

md_status md_get_forces(md_ctx *c, double *force4)
{
    if (!c || !force4) return MD_ERR_ARG;
    return gather_to_host(c, 2, force4, 4 * (size_t)c->n);
}

md_status md_get_energies(md_ctx *c, double *epot)
{
    if (!c || !epot) return MD_ERR_ARG;
    return gather_to_host(c, 3, epot, (size_t)c->n);
}

static md_status scatter_from_host(md_ctx *c, int what, const double *src)
{
    if (what == 0) {
        int cen = 1;
        if (c->batch) {
            size_t o = 0;
            for (int r = 0; r < c->nrep && cen; r++) {
                if (!centered_range(src + 3 * o, c->rep_natom[r], c->reps[r].box)) cen = 0;
                o += (size_t)c->rep_natom[r];
            }
        } else {
            cen = centered_range(src, c->n, c->box) ? 1 : 0;
        }
        if (cen != c->centered && c->gexec) {   /* the step graph holds the old flag */
            cudaGraphExecDestroy(c->gexec);
            c->gexec = nullptr;
        }
        c->centered = cen;
    }
    md_kparams kp = md_make_kparams(c);
    MD_CUDA_TRY(c, cudaMemcpyAsync(c->io_dev, src, sizeof(double) * 3 * (size_t)c->n,
                                   cudaMemcpyHostToDevice, c->stream));
    launch_scatter_in(c, kp, what, c->io_dev);
    return MD_OK;
}

md_status md_set_positions(md_ctx *c, const double *pos3)
{
    if (!c || !pos3) return MD_ERR_ARG;
    md_status s = scatter_from_host(c, 0, pos3);
    if (s != MD_OK) return s;
    s = initial_build(c);
    if (s != MD_OK) return s;
    return refresh_state(c);
}

md_status md_set_velocities(md_ctx *c, const double *vel3)
{
    if (!c || !vel3) return MD_ERR_ARG;
    md_status s = scatter_from_host(c, 1, vel3);
    if (s != MD_OK) return s;
    md_kparams kp = md_make_kparams(c);
    launch_thermo_from_state(c, kp, 0);
    return check_overflow_and_sync(c);
}

md_status md_update_neighbors(md_ctx *c, int force)
{
    if (!c) return MD_ERR_ARG;
    md_kparams kp = md_make_kparams(c);
    if (force) return initial_build(c);
    MD_CUDA_TRY(c, cudaMemsetAsync(&c->st->update, 0, sizeof(int), c->stream));
    launch_check(c, kp);
    launch_rebuild(c, kp, false, false);
    return check_overflow_and_sync(c);
}

md_status md_get_neighbor_list(md_ctx *c, unsigned *nnlist, unsigned *nnlist_max, int pitch, int nmax)
{
    if (!c || !nnlist || !nnlist_max || pitch < c->n || nmax <= 0) return MD_ERR_ARG;
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    const size_t P = c->pitch;
    std::vector<unsigned> nl((size_t)c->cap * P);
    std::vector<int> cnt(P), perm(P);
    MD_CUDA_TRY(c, cudaMemcpy(nl.data(), c->nl, sizeof(unsigned) * nl.size(), cudaMemcpyDeviceToHost));
    MD_CUDA_TRY(c, cudaMemcpy(cnt.data(), c->nl_n, sizeof(int) * P, cudaMemcpyDeviceToHost));
    MD_CUDA_TRY(c, cudaMemcpy(perm.data(), c->perm, sizeof(int) * P, cudaMemcpyDeviceToHost));
    md_status s = MD_OK;
    std::vector<unsigned> row;
    for (int i = 0; i < pitch; i++) nnlist_max[i] = 0;
    for (int si = 0; si < c->n; si++) {
        row.clear();
        for (int k = 0; k < cnt[si]; k++)
            row.push_back((unsigned)perm[nl[(size_t)si * c->cap + k] & MD_INDEX_MASK]);
        std::sort(row.begin(), row.end());
        int o = perm[si];
        nnlist_max[o] = (unsigned)row.size();
        if ((int)row.size() > nmax) s = MD_ERR_LIST_OVERFLOW;
        for (size_t k = 0; k < row.size() && (int)k < nmax; k++) nnlist[o + (size_t)pitch * k] = row[k];
    }
    return s;
}

md_status md_compute_forces(md_ctx *c, int terms, int energy)
{
    if (!c || (terms & ~MD_TERM_ALL)) return MD_ERR_ARG;
    md_kparams kp = md_make_kparams(c);
    launch_forces(c, kp, energy != 0, terms);
    if (energy) launch_thermo_from_state(c, kp, 1);
    return check_overflow_and_sync(c);
}

md_status md_integrate(md_ctx *c, int energy)
{
    if (!c) return MD_ERR_ARG;
    if (c->batch || c->integrator != MD_LEAPFROG)
        return fail(c, MD_ERR_UNSUPPORTED, "md_integrate: leapfrog single systems (velocity Verlet: "
                                           "md_integrate_pre / md_integrate_cor)");
    md_kparams kp = md_make_kparams(c);
    launch_leapfrog(c, kp, energy != 0, 0, 0);
    c->host_step++;
    return check_overflow_and_sync(c);
}

md_status md_integrate_pre(md_ctx *c)
{
    if (!c) return MD_ERR_ARG;
    if (c->batch) return fail(c, MD_ERR_UNSUPPORTED, "md_integrate_pre: single systems");
    md_kparams kp = md_make_kparams(c);
    if (c->integrator == MD_LEAPFROG) {   /* the caller runs velocity Verlet from now on */
        c->integrator = c->enstype == 1 ? MD_NH : MD_VV;
        if (c->gexec) {
            cudaGraphExecDestroy(c->gexec);
            c->gexec = nullptr;
        }
        /* the thermostat's first half step from the current state, as a
         * velocity-Verlet context has it from its creation */
        launch_thermo_from_state(c, kp, 0);
    }
    launch_vv_first(c, kp, 0, 0);
    return check_overflow_and_sync(c);
}

md_status md_integrate_cor(md_ctx *c, int energy)
{
    if (!c) return MD_ERR_ARG;
    if (c->batch || c->integrator == MD_LEAPFROG)
        return fail(c, MD_ERR_UNSUPPORTED, "md_integrate_cor: after md_integrate_pre (single systems)");
    md_kparams kp = md_make_kparams(c);
    launch_vv_second(c, kp, energy != 0);
    c->host_step++;
    return check_overflow_and_sync(c);
}

/* The host copy of the replica table after steps that moved the boxes. */
static md_status sync_reps(md_ctx *c)
{
    if (!c->batch || c->enstype != 2) return MD_OK;
    MD_CUDA_TRY(c, cudaMemcpy(c->reps.data(), c->reps_dev, sizeof(md_rep) * c->nrep, cudaMemcpyDeviceToHost));
    for (int k = 0; k < 3; k++) {   /* the context-wide box: replica 0's */
        c->box[k] = c->reps[0].box[k];
        c->boxi[k] = c->reps[0].boxi[k];
        c->binlen[k] = c->reps[0].binlen[k];
    }
    return MD_OK;
}

static md_status step_body(md_ctx *c, int nsteps, int energy_every, bool mark_start)
{
    if (mark_start) MD_CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
    int left = nsteps;
    while (left > 0) {
        int aligned = energy_every > 0 ? (int)(c->host_step % energy_every == 0) : 1;
        int g = energy_every > 0 ? energy_every : std::min(nsteps, 32);
        if (!aligned || left < g || !c->use_graphs) {
            /* eager steps up to the next aligned step / the remainder */
            int k = left;
            if (energy_every > 0 && !aligned && c->use_graphs) {
                long long next = (c->host_step / energy_every + 1) * energy_every;
                k = (int)std::min<long long>(left, next - c->host_step);
            }
            for (int t = 0; t < k; t++) {
                int en = energy_every > 0 && (c->host_step % energy_every == 0);
                enqueue_steps(c, 1, en);
                c->host_step++;
            }
            left -= k;
            continue;
        }
        int en = energy_every > 0 ? 1 : 0;
        if (!c->gexec || c->gsteps != g || c->genergy != en || c->gpos4 != c->pos4) {
            md_status s = capture_graph(c, g, en);
            if (s != MD_OK) return s;
        }
        while (left >= g && (energy_every == 0 || c->host_step % energy_every == 0)) {
            MD_CUDA_TRY(c, cudaGraphLaunch(c->gexec, c->stream));
            c->host_step += g;
            left -= g;
        }
    }
    MD_CUDA_TRY(c, cudaEventRecord(c->ev1, c->stream));
    MD_CUDA_TRY(c, cudaGetLastError());
    return check_overflow_and_sync(c);
}

/* The arrays a run of steps changes, in the order they are packed into the
 * snapshot: the integrated state and everything a re-sort permutes (the
 * list, cells and sorted bonded lists are rebuilt after a restore). */
struct snap_part {
    void *dev;
    size_t bytes;
};
static std::vector<snap_part> snap_parts(md_ctx *c)
{
    const size_t P = c->pitch;
    std::vector<snap_part> v = {
        {c->st, sizeof(md_devstate)},       {c->x, 3 * P * sizeof(double)},
        {c->v, 3 * P * sizeof(double)},     {c->mass, P * sizeof(double)},
        {c->kick, P * sizeof(double)},      {c->pos4, P * sizeof(float4)},
        {c->type, P * sizeof(int)},         {c->perm, P * sizeof(int)},
        {c->iperm, P * sizeof(int)},        {c->f, 3 * P * sizeof(long long)},
        {c->vir, P * sizeof(float)},        {c->epot, P * sizeof(float)}};
    if (c->batch) {
        v.push_back({c->repst, c->nrep * sizeof(md_repstate)});
        v.push_back({c->racc, 3 * (size_t)c->nrep * sizeof(unsigned long long)});
        v.push_back({c->rep_upd, c->nrep * sizeof(int)});
        v.push_back({c->reps_dev, c->nrep * sizeof(md_rep)});   /* NPT moves the boxes */
    }
    return v;
}

/* Up to MD_SNAP_PARTS device-to-device copies in one launch: blockIdx.y picks
 * the copy, the x blocks stride through it in 16-byte words (every part
 * starts on a 256-byte boundary in both buffers) and 4-byte words for a
 * tail (every part is a multiple of 4 bytes). */
#define MD_SNAP_PARTS 16
struct snap_copies {
    const char *src[MD_SNAP_PARTS];
    char *dst[MD_SNAP_PARTS];
    unsigned long long bytes[MD_SNAP_PARTS];
};
__global__ void k_snapshot(snap_copies cp)
{
    const int k = blockIdx.y;
    const unsigned long long nb = cp.bytes[k], n16 = nb / 16;
    const uint4 *s16 = (const uint4 *)cp.src[k];
    uint4 *d16 = (uint4 *)cp.dst[k];
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n16; i += stride)
        d16[i] = s16[i];
    if (blockIdx.x == 0)
        for (unsigned long long i = n16 * 4 + threadIdx.x; i < nb / 4; i += blockDim.x)
            ((unsigned *)cp.dst[k])[i] = ((const unsigned *)cp.src[k])[i];
}

/* Stream-ordered device copies of the state into the snapshot (or back),
 * one kernel launch for all parts. */
static md_status snapshot(md_ctx *c, bool save)
{
    std::vector<snap_part> parts = snap_parts(c);
    size_t total = 0;
    for (const snap_part &p : parts) total += (p.bytes + 255) / 256 * 256;
    if (save && c->snap_bytes < total) {
        if (c->snap) cudaFree(c->snap);
        c->snap = nullptr;
        c->snap_bytes = 0;
        MD_CUDA_TRY(c, cudaMalloc(&c->snap, total));
        c->snap_bytes = total;
    }
    if (save) {
        c->snap_p4 = c->pos4;
        c->snap_p4alt = c->pos4_alt;
        c->snap_host_step = c->host_step;
    } else {
        c->pos4 = c->snap_p4;
        c->pos4_alt = c->snap_p4alt;
        c->host_step = c->snap_host_step;
        parts = snap_parts(c);   /* pos4 is the buffer current at the save */
    }
    if (parts.size() > MD_SNAP_PARTS) return fail(c, MD_ERR_ARG, "snapshot: too many parts");
    snap_copies cp;
    memset(&cp, 0, sizeof(cp));
    size_t off = 0, maxb = 0;
    for (size_t k = 0; k < parts.size(); k++) {
        char *s = (char *)c->snap + off;
        cp.src[k] = save ? (const char *)parts[k].dev : s;
        cp.dst[k] = save ? s : (char *)parts[k].dev;
        cp.bytes[k] = parts[k].bytes;
        maxb = std::max(maxb, parts[k].bytes);
        off += (parts[k].bytes + 255) / 256 * 256;
    }
    const int bx = (int)std::min<size_t>(std::max<size_t>((maxb / 16 + 255) / 256, 1), 512);
    k_snapshot<<<dim3(bx, (unsigned)parts.size()), 256, 0, c->stream>>>(cp);
    MD_CUDA_TRY(c, cudaGetLastError());
    return MD_OK;
}

/* NPT: lay the cells of every replica of the batch out again for its
 * current box (the same rule as at creation: cells of at least 1.03 times
 * half the list radius), reallocate the cell tables when their total
 * changes, and rebuild every replica's list on the new grid. */
static md_status regrid_batch(md_ctx *c)
{
    std::vector<int> rank, lin, crep;
    const std::vector<md_rep> reps_before = c->reps;
    int cell0 = 0;
    for (int r = 0; r < c->nrep; r++) {
        md_rep &R = c->reps[r];
        const float rl = 2.0f * R.rl_half;
        cell_grid g;
        make_cell_grid(R.box, R.npt ? rl * 1.03f : rl, g);
        int nst = 1;
        for (int k = 0; k < 3; k++) nst *= g.stencil[k] < 0 ? g.ncell[k] : 2 * g.stencil[k] + 1;
        if (nst > 128) {
            c->reps = reps_before;
            return fail(c, MD_ERR_UNSUPPORTED, "NPT regrid: stencil too large");
        }
        for (int k = 0; k < 3; k++) {
            R.ncell[k] = g.ncell[k];
            R.stencil[k] = g.stencil[k];
            R.binlen[k] = g.binlen[k];
        }
        R.cell_shift = md_cell_shift(R.stencil, R.binlen, R.box);
        R.cell0 = cell0;
        R.ncells = g.ncells;
        for (int k = 0; k < g.ncells; k++) {
            rank.push_back(cell0 + g.rank[k]);
            lin.push_back(g.lin[k]);
            crep.push_back(r);
        }
        cell0 += g.ncells;
    }
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (cell0 != c->ncells) {
        /* the new tables first: on a failed allocation the context keeps
         * its old grid (whose box check then reports MD_ERR_BOX) */
        int **arr[] = {&c->cell_rank, &c->cell_lin, &c->cell_count, &c->cell_start, &c->cell_fill, &c->cell_work,
                       &c->crep};
        constexpr int NA = sizeof(arr) / sizeof(arr[0]);
        int *fresh[NA] = {};
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < NA && e == cudaSuccess; k++)
            e = dalloc(&fresh[k], (size_t)cell0 + (arr[k] == &c->cell_start ? 1 : 0));
        if (e != cudaSuccess) {
            for (int *q : fresh) cudaFree(q);
            (void)cudaGetLastError();
            c->reps = reps_before;
            return fail(c, MD_ERR_CUDA, std::string("NPT regrid: ") + cudaGetErrorString(e));
        }
        for (int k = 0; k < NA; k++) {
            cudaFree(*arr[k]);
            *arr[k] = fresh[k];
        }
        c->ncells = cell0;
    }
    std::vector<int> zeros(cell0, 0);
    MD_CUDA_TRY(c, cudaMemcpy(c->cell_rank, rank.data(), sizeof(int) * cell0, cudaMemcpyHostToDevice));
    MD_CUDA_TRY(c, cudaMemcpy(c->cell_lin, lin.data(), sizeof(int) * cell0, cudaMemcpyHostToDevice));
    MD_CUDA_TRY(c, cudaMemcpy(c->crep, crep.data(), sizeof(int) * cell0, cudaMemcpyHostToDevice));
    MD_CUDA_TRY(c, cudaMemcpy(c->cell_count, zeros.data(), sizeof(int) * cell0, cudaMemcpyHostToDevice));
    MD_CUDA_TRY(c, cudaMemcpy(c->cell_fill, zeros.data(), sizeof(int) * cell0, cudaMemcpyHostToDevice));
    MD_CUDA_TRY(c, cudaMemcpy(c->reps_dev, c->reps.data(), sizeof(md_rep) * c->nrep, cudaMemcpyHostToDevice));
    for (int k = 0; k < 3; k++) {
        c->ncell[k] = c->reps[0].ncell[k];
        c->binlen[k] = c->reps[0].binlen[k];
        c->stencil[k] = c->reps[0].stencil[k];
    }
    if (c->gexec) {   /* the step graphs hold the old cell count */
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    c->regrids++;
    return initial_build(c);
}

/* NPT: whether a replica's cells have come within half the grid's 3%
 * margin of half its list radius (regrid before they can fall below it),
 * or its box has grown enough for one more cell with 1% to spare (fewer
 * atoms per stencil; the 4% between the two keeps a box that fluctuates
 * about one size from regridding back and forth). */
static bool regrid_due(const md_ctx *c)
{
    if (!c->batch || c->enstype != 2) return false;
    for (const md_rep &R : c->reps) {
        if (!R.npt) continue;
        for (int k = 0; k < 3; k++) {
            if (R.stencil[k] >= 0 && R.binlen[k] < R.rl_half * 1.015f) return true;
            const int fit = (int)floorf(R.box[k] / (R.rl_half * 1.03f * 1.0001f * 1.01f));
            if (std::min(fit, 1024) > R.ncell[k]) return true;
        }
    }
    return false;
}

static md_status md_step_impl(md_ctx *c, int nsteps, int energy_every, bool mark_start);

/* NPT batches run in chunks of at most MD_NPT_CHUNK steps (a whole
 * multiple of energy_every when that fits, so that the chunks stay aligned
 * with the energy steps), each ending with the regrid check: at the
 * per-step clamp of the box scale (1e-4) a chunk shrinks a box by at most
 * 1.3%, less than the 1.5% left between the regrid threshold and the
 * limit.  Energy steps are multiples of energy_every counted from the
 * context's first step, so a chunk boundary never moves them. */
#define MD_NPT_CHUNK 128
md_status md_step(md_ctx *c, int nsteps, int energy_every)
{
    if (!c || nsteps < 0 || energy_every < 0) return MD_ERR_ARG;
    if (!(c->batch && c->enstype == 2)) return md_step_impl(c, nsteps, energy_every, true);
    const int chunk = (energy_every > 0 && energy_every <= MD_NPT_CHUNK)
                          ? MD_NPT_CHUNK / energy_every * energy_every
                          : MD_NPT_CHUNK;
    int done = 0;
    do {
        const int k = std::min(chunk, nsteps - done);
        md_status s = md_step_impl(c, k, energy_every, done == 0);
        if (s == MD_OK && regrid_due(c)) s = regrid_batch(c);
        if (s != MD_OK) return s;
        done += k;
    } while (done < nsteps);
    return MD_OK;
}

/* A list overflow inside a run of steps truncates rows, so every step after
 * the rebuild that overflowed is wrong.  md_step therefore saves the state
 * on the device when it starts (a few device-to-device copies, ~170 B per
 * atom) and, when the run ends with an overflow, restores it, grows the
 * list to 5/4 of the longest row plus 16, rebuilds it at the restored
 * positions (forces recomputed for velocity Verlet) and runs the same steps
 * again, up to three times. */
static md_status md_step_impl(md_ctx *c, int nsteps, int energy_every, bool mark_start)
{
    if (!c->overflow_retry || nsteps == 0) {
        md_status s0 = step_body(c, nsteps, energy_every, mark_start);
        return s0 == MD_OK ? sync_reps(c) : s0;
    }
    /* the call's device time (md_last_step_ms) includes the snapshot */
    if (mark_start) MD_CUDA_TRY(c, cudaEventRecord(c->ev0, c->stream));
    md_status s = snapshot(c, true);
    if (s != MD_OK) return s;
    s = step_body(c, nsteps, energy_every, false);
    for (int tries = 0; s == MD_ERR_LIST_OVERFLOW && tries < 3; tries++) {
        md_devstate h;
        MD_CUDA_TRY(c, cudaMemcpy(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost));
        const int cap = ((h.list_overflow * 5 / 4 + 16) + 31) / 32 * 32;
        s = snapshot(c, false);   /* the saved state has no overflow recorded */
        if (s == MD_OK) s = sync_reps(c);
        if (s != MD_OK) return s;
        if (c->gexec) {           /* the step graph holds the old capacity */
            cudaGraphExecDestroy(c->gexec);
            c->gexec = nullptr;
        }
        s = alloc_list(c, std::max(cap, c->cap));
        if (s == MD_OK) s = initial_build(c);
        if (s == MD_OK) s = refresh_state(c);
        if (s != MD_OK) return s;
        c->regrows++;
        s = step_body(c, nsteps, energy_every, false);
    }
    if (s == MD_OK) s = sync_reps(c);
    return s;
}

md_status md_last_step_ms(md_ctx *c, float *ms)
{
    if (!c || !ms) return MD_ERR_ARG;
    MD_CUDA_TRY(c, cudaEventSynchronize(c->ev1));
    MD_CUDA_TRY(c, cudaEventElapsedTime(ms, c->ev0, c->ev1));
    return MD_OK;
}

md_status md_get_thermo(md_ctx *c, md_thermo *out)
{
    if (!c || !out) return MD_ERR_ARG;
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    md_devstate h;
    MD_CUDA_TRY(c, cudaMemcpy(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost));
    if (h.step == 0) {
        memset(out, 0, sizeof(*out));
        out->ke = h.ke;
        out->temper = 2.0 * h.ke / (md_ndf(c) * 8.314e-3);
        out->pe = h.pe;
        out->virial = h.virial;
        out->conserved = h.ke + h.pe;
        out->builds = h.builds;
        out->lambda = 1.0;
        return MD_OK;
    }
    MD_CUDA_TRY(c, cudaMemcpy(out, c->rec + (h.step - 1) % c->rec_cap, sizeof(md_thermo),
                              cudaMemcpyDeviceToHost));
    return MD_OK;
}

md_status md_get_thermo_history(md_ctx *c, md_thermo *out, int n, int *got)
{
    if (!c || !out || n < 0 || !got) return MD_ERR_ARG;
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    md_devstate h;
    MD_CUDA_TRY(c, cudaMemcpy(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost));
    long long avail = std::min<long long>(h.step, c->rec_cap);
    int k = (int)std::min<long long>(avail, n);
    /* the last k records of the ring: at most two contiguous ranges */
    int t = 0;
    while (t < k) {
        const int r = (int)((h.step - k + t) % c->rec_cap);
        const int len = std::min(k - t, c->rec_cap - r);
        MD_CUDA_TRY(c, cudaMemcpyAsync(out + t, c->rec + r, sizeof(md_thermo) * (size_t)len,
                                       cudaMemcpyDeviceToHost, c->stream));
        t += len;
    }
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    *got = k;
    return MD_OK;
}

md_status md_get_replica_history(md_ctx *c, double *out, int n, int *got)
{
    if (!c || !out || n < 0 || !got) return MD_ERR_ARG;
    if (!c->batch) {
        c->last_error = "md_get_replica_history: not a batch context";
        return MD_ERR_ARG;
    }
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    md_devstate h;
    MD_CUDA_TRY(c, cudaMemcpy(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost));
    const long long avail = std::min<long long>(h.step, c->rec_cap);
    const int k = (int)std::min<long long>(avail, n);
    const size_t row = (size_t)3 * c->nrep;   /* doubles per step */
    int t = 0;
    while (t < k) {
        const int r = (int)((h.step - k + t) % c->rec_cap);
        const int len = std::min(k - t, c->rec_cap - r);
        MD_CUDA_TRY(c, cudaMemcpyAsync(out + (size_t)t * row, c->rep_hist + (size_t)r * row,
                                       sizeof(double) * row * (size_t)len, cudaMemcpyDeviceToHost, c->stream));
        t += len;
    }
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    *got = k;
    return MD_OK;
}

md_status md_run_host(md_ctx *c, double *pos3, double *vel3, int nsteps, int energy_every,
                      md_thermo *records)
{
    if (!c || !pos3 || !vel3 || nsteps < 0) return MD_ERR_ARG;
    if (nsteps > c->rec_cap && records) return MD_ERR_ARG;
    /* The launches of md_set_positions and md_set_velocities (upload, forced
     * build, forces and thermodynamic state) with one synchronisation; on a
     * list overflow those two calls run again and grow the list. */
    md_status s = scatter_from_host(c, 0, pos3);
    if (s != MD_OK) return s;
    md_kparams kp = md_make_kparams(c);
    launch_rebuild(c, kp, true, true);
    launch_forces(c, kp, true, MD_TERM_ALL);
    launch_thermo_from_state(c, kp, 1);
    s = scatter_from_host(c, 1, vel3);
    if (s != MD_OK) return s;
    launch_thermo_from_state(c, kp, 0);
    s = check_overflow_and_sync(c);
    if (s == MD_ERR_LIST_OVERFLOW) {
        s = md_set_positions(c, pos3);
        if (s == MD_OK) s = md_set_velocities(c, vel3);
    }
    if (s == MD_OK) s = md_step(c, nsteps, energy_every);
    if (s == MD_OK && records) {
        int got = 0;
        s = md_get_thermo_history(c, records, nsteps, &got);
    }
    if (s != MD_OK) return s;
    /* positions, then velocities, through the staging buffer in stream order */
    kp = md_make_kparams(c);
    const size_t bytes = sizeof(double) * 3 * (size_t)c->n;
    launch_gather_out(c, kp, 0, c->io_dev);
    MD_CUDA_TRY(c, cudaMemcpyAsync(pos3, c->io_dev, bytes, cudaMemcpyDeviceToHost, c->stream));
    launch_gather_out(c, kp, 1, c->io_dev);
    MD_CUDA_TRY(c, cudaMemcpyAsync(vel3, c->io_dev, bytes, cudaMemcpyDeviceToHost, c->stream));
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return MD_OK;
}

md_status md_write_cfg(md_ctx *c, const char *path)
{
    if (!c || !path) return MD_ERR_ARG;
    if (c->batch) return fail(c, MD_ERR_UNSUPPORTED, "md_write_cfg: a batch holds several boxes");
    std::vector<double> p(3 * (size_t)c->n), v(3 * (size_t)c->n);
    md_status s = md_get_positions(c, p.data());
    if (s == MD_OK) s = md_get_velocities(c, v.data());
    if (s != MD_OK) return s;
    FILE *fo = fopen(path, "w");
    if (!fo) return fail(c, MD_ERR_IO, std::string("cannot write ") + path);
    fprintf(fo, "%d %d\n", c->n, 1);
    fprintf(fo, "%.9g %.9g %.9g\n", c->box[0], c->box[1], c->box[2]);
    for (int i = 0; i < c->n; i++) {
        fprintf(fo, "%d %d %.9g\n", i + 1, c->itype[i] + 1, c->charge[i]);
        fprintf(fo, "%.17g %.17g %.17g\n", p[3 * i], p[3 * i + 1], p[3 * i + 2]);
        fprintf(fo, "%.17g %.17g %.17g\n", v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    }
    fclose(fo);
    return MD_OK;
}

md_status md_write_xyz(md_ctx *c, const char *path, int append)
{
    if (!c || !path) return MD_ERR_ARG;
    std::vector<double> p(3 * (size_t)c->n);
    md_status s = md_get_positions(c, p.data());
    if (s != MD_OK) return s;
    FILE *fo = fopen(path, append ? "a" : "w");
    if (!fo) return fail(c, MD_ERR_IO, std::string("cannot write ") + path);
    fprintf(fo, "%d\n", c->n);
    if (c->batch)
        fprintf(fo, "step %lld replicas %d\n", c->host_step, c->nrep);
    else
        fprintf(fo, "step %lld box %.9g %.9g %.9g\n", c->host_step, c->box[0], c->box[1], c->box[2]);
    for (int i = 0; i < c->n; i++) {
        const int t = c->itype[i];
        if (t < (int)c->type_names.size())
            fprintf(fo, "%s", c->type_names[t].c_str());
        else
            fprintf(fo, "T%d", t + 1);
        fprintf(fo, " %.17g %.17g %.17g\n", p[3 * i], p[3 * i + 1], p[3 * i + 2]);
    }
    const int bad = ferror(fo);
    fclose(fo);
    return bad ? fail(c, MD_ERR_IO, std::string("writing ") + path) : MD_OK;
}

/* Restart file: magic, version, atoms, step, then FP64 positions and
 * velocities as stored (original order) and the thermodynamic state. */
static const char MD_RESTART_MAGIC[8] = {'M', 'D', 'G', 'B', '3', 'R', 'S', 'T'};
struct md_restart_state {
    long long step;
    int builds, pad;
    double temper, ke, pe, virial, xi, eta, xi_a, eta_a, vscale, lambda, lam_next, kick_scale;
    md_thermo last;   /* the record of the last step (md_get_thermo) */
};

md_status md_write_restart(md_ctx *c, const char *path)
{
    if (!c || !path) return MD_ERR_ARG;
    if (c->batch) return fail(c, MD_ERR_UNSUPPORTED, "md_write_restart: single systems");
    const size_t n3 = 3 * (size_t)c->n;
    std::vector<double> p(n3), v(n3);
    md_status s = md_get_positions(c, p.data());
    if (s != MD_OK) return s;
    md_kparams kp = md_make_kparams(c);
    launch_gather_out(c, kp, 4, c->io_dev);
    MD_CUDA_TRY(c, cudaMemcpyAsync(v.data(), c->io_dev, sizeof(double) * n3, cudaMemcpyDeviceToHost, c->stream));
    md_devstate h;
    MD_CUDA_TRY(c, cudaMemcpyAsync(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    md_restart_state r;
    memset(&r, 0, sizeof(r));
    r.step = c->host_step;
    r.builds = h.builds;
    r.temper = h.temper;
    r.ke = h.ke;
    r.pe = h.pe;
    r.virial = h.virial;
    r.xi = h.xi;
    r.eta = h.eta;
    r.xi_a = h.xi_a;
    r.eta_a = h.eta_a;
    r.vscale = h.vscale;
    r.lambda = h.lambda;
    r.lam_next = h.lam_next;
    r.kick_scale = h.kick_scale;
    if (h.step > 0)
        MD_CUDA_TRY(c, cudaMemcpy(&r.last, c->rec + (h.step - 1) % c->rec_cap, sizeof(md_thermo),
                                  cudaMemcpyDeviceToHost));
    FILE *fo = fopen(path, "wb");
    if (!fo) return fail(c, MD_ERR_IO, std::string("cannot write ") + path);
    const int head[2] = {1, c->n};
    bool ok = fwrite(MD_RESTART_MAGIC, 1, 8, fo) == 8 && fwrite(head, sizeof(int), 2, fo) == 2 &&
              fwrite(&r, sizeof(r), 1, fo) == 1 && fwrite(p.data(), sizeof(double), n3, fo) == n3 &&
              fwrite(v.data(), sizeof(double), n3, fo) == n3;
    ok = (fclose(fo) == 0) && ok;
    return ok ? MD_OK : fail(c, MD_ERR_IO, std::string("writing ") + path);
}

md_status md_read_restart(md_ctx *c, const char *path)
{
    if (!c || !path) return MD_ERR_ARG;
    if (c->batch) return fail(c, MD_ERR_UNSUPPORTED, "md_read_restart: single systems");
    FILE *fi = fopen(path, "rb");
    if (!fi) return fail(c, MD_ERR_IO, std::string("cannot read ") + path);
    char magic[8];
    int head[2] = {0, 0};
    md_restart_state r;
    const size_t n3 = 3 * (size_t)c->n;
    std::vector<double> p(n3), v(n3);
    bool ok = fread(magic, 1, 8, fi) == 8 && !memcmp(magic, MD_RESTART_MAGIC, 8) &&
              fread(head, sizeof(int), 2, fi) == 2 && head[0] == 1 && head[1] == c->n &&
              fread(&r, sizeof(r), 1, fi) == 1 && fread(p.data(), sizeof(double), n3, fi) == n3 &&
              fread(v.data(), sizeof(double), n3, fi) == n3;
    fclose(fi);
    if (!ok) return fail(c, MD_ERR_PARSE, std::string(path) + ": not a restart file of this system");
    md_status s = md_set_positions(c, p.data());
    if (s == MD_OK) s = md_set_velocities(c, v.data());
    if (s != MD_OK) return s;
    md_devstate h;
    MD_CUDA_TRY(c, cudaMemcpy(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost));
    h.step = r.step;
    h.builds = r.builds;
    h.temper = r.temper;
    h.ke = r.ke;
    h.pe = r.pe;
    h.virial = r.virial;
    h.xi = r.xi;
    h.eta = r.eta;
    h.xi_a = r.xi_a;
    h.eta_a = r.eta_a;
    h.vscale = r.vscale;
    h.lambda = r.lambda;
    h.lam_next = r.lam_next;
    h.kick_scale = r.kick_scale;
    MD_CUDA_TRY(c, cudaMemcpy(c->st, &h, sizeof(h), cudaMemcpyHostToDevice));
    if (r.step > 0)
        MD_CUDA_TRY(c, cudaMemcpy(c->rec + (r.step - 1) % c->rec_cap, &r.last, sizeof(md_thermo),
                                  cudaMemcpyHostToDevice));
    c->host_step = r.step;
    return MD_OK;
}

md_status md_get_info(md_ctx *c, md_info *out)
{
    if (!c || !out) return MD_ERR_ARG;
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    md_devstate h;
    MD_CUDA_TRY(c, cudaMemcpy(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost));
    std::vector<int> cnt(c->pitch);
    MD_CUDA_TRY(c, cudaMemcpy(cnt.data(), c->nl_n, sizeof(int) * c->pitch, cudaMemcpyDeviceToHost));
    out->natom = c->n;
    out->pitch = c->pitch;
    out->capacity = c->cap;
    for (int k = 0; k < 3; k++) {
        out->ncell[k] = c->ncell[k];
        out->stencil[k] = c->stencil[k];
        out->binlen[k] = c->binlen[k];
    }
    out->pair_threads_per_atom = c->pair_tpa;
    out->pair_entries_per_lane = md_pair_depth(c);
    out->positions_centered = c->centered;
    out->fused_step = md_can_fuse(c) ? 1 : 0;
    out->rebuild_inline = (c->rebuild_inline && !c->batch) ? 1 : 0;
    out->list_regrows = c->regrows;
    out->cell_regrids = c->regrids;
    out->list_threads_per_atom = c->list_tpa;
    out->builds = h.builds;
    out->max_neighbors = *std::max_element(cnt.begin(), cnt.begin() + c->n);
    /* in a step graph without a rebuild: pair, bonded (if any), integrator
     * (leapfrog: one kernel; VV: two); a rebuild adds 9 kernels */
    out->kernels_per_step = md_can_fuse(c) ? 1
                                           : 1 + ((c->has_bonds || c->has_angles) ? 1 : 0) +
                                                 (c->integrator == MD_LEAPFROG ? 1 : 2);
    /* PME: spread, solve, gather and (with exclusions) the correction, plus
     * the kernels of cuFFT's two transforms, which are not counted */
    if (c->pme.on) out->kernels_per_step += 3 + c->pme.excl;
    for (int k = 0; k < 3; k++) out->pme_grid[k] = c->pme.K[k];
    /* single system: one cooperative kernel, or key, scan, scatter, order,
     * permute, copyback, remap (with bonds or angles), list, clear; batch:
     * flag (forced builds only, not counted), key, scan, scatter, order,
     * permute, copyback, remap (with bonds or angles), list, clear */
    out->kernels_per_rebuild = md_rebuild_coop(c) ? 1 : !(c->has_bonds || c->has_angles) ? 8 : 9;
    out->kernels_per_graph = c->integrator == MD_LEAPFROG ? 1 : 0;
    if (c->rebuild_inline && !c->batch) {   /* the passes run (and return) in every step */
        out->kernels_per_step += out->kernels_per_rebuild;
        out->kernels_per_rebuild = 0;
        out->kernels_per_graph = 0;
    }
    return MD_OK;
}

md_status md_get_order(md_ctx *c, int *perm)
{
    if (!c || !perm) return MD_ERR_ARG;
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    MD_CUDA_TRY(c, cudaMemcpy(perm, c->perm, sizeof(int) * c->n, cudaMemcpyDeviceToHost));
    return MD_OK;
}

md_status md_get_cell_ranks(md_ctx *c, int *rank)
{
    if (!c || !rank) return MD_ERR_ARG;
    MD_CUDA_TRY(c, cudaMemcpy(rank, c->cell_rank, sizeof(int) * c->ncells, cudaMemcpyDeviceToHost));
    return MD_OK;
}

md_status md_set_type_exclusions(md_ctx *c, const unsigned *mask)
{
    if (!c || !mask) return MD_ERR_ARG;
    if (c->pme.on)
        return fail(c, MD_ERR_UNSUPPORTED, "md_set_type_exclusions: the reciprocal Ewald sum (md_set_pme) "
                                           "takes no type exclusions");
    unsigned m[MD_MAXTYPE] = {0};
    for (int a = 0; a < c->ntype; a++)
        for (int b = 0; b < c->ntype; b++)
            if (((mask[a] >> b) & 1u) || ((mask[b] >> a) & 1u)) m[a] |= 1u << b;
    memcpy(c->type_excl_mask, m, sizeof(m));
    MD_CUDA_TRY(c, cudaMemcpyAsync(c->type_mask_dev, m, sizeof(m), cudaMemcpyHostToDevice, c->stream));
    md_status s = initial_build(c);
    if (s != MD_OK) return s;
    return refresh_state(c);
}

md_status md_set_pme(md_ctx *c, int k0, int k1, int k2)
{
    if (!c) return MD_ERR_ARG;
    const int K[3] = {k0, k1, k2};
    const bool off = k0 == 0 && k1 == 0 && k2 == 0;
    if (!off) {
        for (int d = 0; d < 3; d++)
            if (K[d] < 16 || K[d] % 8 || K[d] > 2048)
                return fail(c, MD_ERR_ARG, "md_set_pme: grid points per axis must be multiples of 8 in [16, 2048]");
        if (c->lkspace != 2)
            return fail(c, MD_ERR_UNSUPPORTED, "md_set_pme: needs the Ewald real-space term (lkspace 2)");
        if (c->batch)
            return fail(c, MD_ERR_UNSUPPORTED, "md_set_pme: single systems only");
        if (c->fp64) return fail(c, MD_ERR_UNSUPPORTED, "md_set_pme: not in the FP64 mode");
        for (int a = 0; a < MD_MAXTYPE; a++)
            if (c->type_excl_mask[a])
                return fail(c, MD_ERR_UNSUPPORTED, "md_set_pme: the context has type exclusions");
    }
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (c->gexec) {   /* the step graphs hold the force kernels they were captured with */
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    md_status s = pme_setup(c, K);
    if (s != MD_OK) return s;
    return refresh_state(c);   /* the forces (and record) of the current state with the new sum */
}

/* Builds so far (synchronises the stream). */
static md_status read_builds(md_ctx *c, int *builds)
{
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    md_devstate h;
    MD_CUDA_TRY(c, cudaMemcpy(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost));
    *builds = h.builds;
    return MD_OK;
}

md_status md_autotune(md_ctx *c, int *pair_tpa, int *list_tpa)
{
    if (!c) return MD_ERR_ARG;
    const int lt[] = {0, 4, 8, 16};
    float best = 1e30f;
    int bp = c->pair_tpa, bl = c->list_tpa, bf = 0;
    c->fuse_step = 0;
    /* best of three timings of 20 launches per candidate (lanes per atom,
     * entries per lane and batch): robust to a slow first launch and to other
     * work on the device. */
    const int combos[][2] = {{2, 0}, {4, 0}, {4, 4}, {8, 0}, {8, 2}, {16, 0}, {16, 1}};
    std::vector<std::pair<float, int>> ranked;   /* (ms, combo) */
    for (int q = 0; q < (int)(sizeof(combos) / sizeof(combos[0])); q++) {
        c->pair_tpa = combos[q][0];
        c->pair_depth = combos[q][1];
        float ms = 0.0f, m2 = 1e30f;
        md_status s = md_time_pair(c, 5, &ms);
        for (int rep = 0; rep < 3 && s == MD_OK; rep++) {
            s = md_time_pair(c, 20, &ms);
            m2 = std::min(m2, ms);
        }
        if (s != MD_OK) return s;
        ranked.push_back({m2, q});
    }
    std::sort(ranked.begin(), ranked.end());
    int bq = ranked[0].second;
    c->pair_tpa = combos[bq][0];
    c->pair_depth = combos[bq][1];
    /* the step graph: separate or (leapfrog without bonded terms) fused pair
     * and integrator kernels, the rebuild behind a conditional node or inline
     * (single systems), for the three fastest pair settings (the fused
     * kernel's own ranking may differ); each combination timed as it runs,
     * 96 steps after 32 of warm-up, less the list builds that fell in the
     * window at the measured cost of one (the system advances 128 steps per
     * combination) */
    int bi = 0;
    c->fuse_step = 1;
    const int nf = md_can_fuse(c) ? 2 : 1, ni = c->batch ? 1 : 2;
    if (nf * ni > 1) {   /* a batch has one choice: it keeps its state */
        float t_rb = 0.0f;
        md_status s = md_time_rebuild(c, 3, &t_rb);
        if (s != MD_OK) return s;
        float tbest = 1e30f;
        for (int cand = 0; cand < std::min(3, (int)ranked.size()); cand++)
        for (int fz = 0; fz < nf; fz++)
            for (int inl = 0; inl < ni; inl++) {
                const int q = ranked[cand].second;
                c->pair_tpa = combos[q][0];
                c->pair_depth = combos[q][1];
                c->fuse_step = fz;
                c->rebuild_inline = inl;
                if (c->gexec) {
                    cudaGraphExecDestroy(c->gexec);
                    c->gexec = nullptr;
                }
                s = md_step(c, 32, 0);
                int b0 = 0, b1 = 0;
                float ms = 0.0f;
                if (s == MD_OK) s = read_builds(c, &b0);
                if (s == MD_OK) s = md_step(c, 96, 0);
                if (s == MD_OK) s = md_last_step_ms(c, &ms);
                if (s == MD_OK) s = read_builds(c, &b1);
                if (s != MD_OK) return s;
                const float t = ms - (float)(b1 - b0) * t_rb;
                if (t < tbest) { tbest = t; bf = fz; bi = inl; bq = q; }
            }
    }
    bp = combos[bq][0];
    c->pair_tpa = bp;
    c->pair_depth = combos[bq][1];
    c->fuse_step = bf;
    c->rebuild_inline = bi;
    best = 1e30f;
    for (int t : lt) {
        if (c->batch && t != 0) continue;   /* batches build one warp per cell */
        c->list_tpa = t;
        float ms = 0.0f, m2 = 1e30f;
        md_status s = md_time_rebuild(c, 2, &ms);
        for (int rep = 0; rep < 3 && s == MD_OK; rep++) {
            s = md_time_rebuild(c, 5, &ms);
            m2 = std::min(m2, ms);
        }
        if (s != MD_OK) return s;
        if (m2 < best) { best = m2; bl = t; }
    }
    c->list_tpa = bl;
    if (c->gexec) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    if (pair_tpa) *pair_tpa = bp;
    if (list_tpa) *list_tpa = bl;
    return MD_OK;
}

md_status md_set_barostat(md_ctx *c, double press_bar, double tau_p_fs, double compressibility_per_bar)
{
    if (!c || tau_p_fs <= 0 || compressibility_per_bar < 0) return MD_ERR_ARG;
    if (!c->batch || c->enstype != 2) {
        c->last_error = "md_set_barostat: not an NPT context";
        return MD_ERR_ARG;
    }
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    md_status s = sync_reps(c);
    if (s != MD_OK) return s;
    c->baro[0] = press_bar;
    c->baro[1] = tau_p_fs;
    c->baro[2] = compressibility_per_bar;
    apply_barostat(c);
    MD_CUDA_TRY(c, cudaMemcpy(c->reps_dev, c->reps.data(), sizeof(md_rep) * c->nrep, cudaMemcpyHostToDevice));
    return MD_OK;
}

md_status md_get_replica_box(md_ctx *c, double *box3, double *pressure_bar, int nrep)
{
    if (!c || !box3 || nrep < 1) return MD_ERR_ARG;
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (!c->batch) {
        for (int k = 0; k < 3; k++) box3[k] = (double)c->box[k];
        if (pressure_bar) pressure_bar[0] = 0.0;
        return MD_OK;
    }
    std::vector<md_rep> reps(c->nrep);
    std::vector<md_repstate> rs(c->nrep);
    MD_CUDA_TRY(c, cudaMemcpy(reps.data(), c->reps_dev, sizeof(md_rep) * c->nrep, cudaMemcpyDeviceToHost));
    MD_CUDA_TRY(c, cudaMemcpy(rs.data(), c->repst, sizeof(md_repstate) * c->nrep, cudaMemcpyDeviceToHost));
    for (int r = 0; r < std::min(nrep, c->nrep); r++) {
        for (int k = 0; k < 3; k++) box3[3 * r + k] = reps[r].boxd[k];
        if (pressure_bar) pressure_bar[r] = rs[r].pressure * MD_BAR;
    }
    return MD_OK;
}

md_status md_debug_list_capacity(md_ctx *c, int capacity, int retry)
{
    if (!c || capacity < 32 || capacity % 32) return MD_ERR_ARG;
    MD_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (c->gexec) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    md_status s = alloc_list(c, capacity);
    if (s != MD_OK) return s;
    const int one = 1;
    MD_CUDA_TRY(c, cudaMemcpy(&c->st->update, &one, sizeof(int), cudaMemcpyHostToDevice));
    if (c->batch) {   /* every replica rebuilds */
        std::vector<int> ones(c->nrep, 1);
        MD_CUDA_TRY(c, cudaMemcpy(c->rep_upd, ones.data(), sizeof(int) * c->nrep, cudaMemcpyHostToDevice));
    }
    c->overflow_retry = retry ? 1 : 0;
    return MD_OK;
}

md_status md_set_precision(md_ctx *c, int bits)
{
    if (!c || (bits != 32 && bits != 64)) return MD_ERR_ARG;
    if (bits == 64 && c->enstype == 2) {
        c->last_error = "md_set_precision: the FP64 mode takes a fixed box (no NPT)";
        return MD_ERR_UNSUPPORTED;
    }
    if (bits == 64 && c->pme.on)
        return fail(c, MD_ERR_UNSUPPORTED, "md_set_precision: the FP64 mode has no reciprocal Ewald sum");
    if (bits == 64 && !c->p64_dev) {
        const int nm = c->batch ? c->nrep : 1;
        std::vector<md_p64> h(nm);
        for (int r = 0; r < nm; r++) {
            if (c->batch) {
                const md_rep &R = c->reps[r];
                h[r] = md_make_p64(c->lkspace, R.rcutsq, R.reacf, c->rep_alfa[r], R.box);
            } else {
                h[r] = md_make_p64(c->lkspace, c->rcutsq, c->reacf, c->alfa, c->box);
            }
        }
        MD_CUDA_TRY(c, dalloc(&c->p64_dev, (size_t)nm));
        MD_CUDA_TRY(c, cudaMemcpy(c->p64_dev, h.data(), sizeof(md_p64) * nm, cudaMemcpyHostToDevice));
    }
    const int v = bits == 64 ? 1 : 0;
    if (v == c->fp64) return MD_OK;
    c->fp64 = v;
    if (c->gexec) {   /* graphs hold the kernels they were captured with */
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    /* the forces (and record) of the current state in the new precision */
    return refresh_state(c);
}

md_status md_debug_rebuild_barrier(md_ctx *c, double timeout_ms, int drop_block)
{
    if (!c || timeout_ms < 0.0 || drop_block < -1) return MD_ERR_ARG;
    c->dbg_bar_ns = (unsigned long long)(timeout_ms * 1e6);
    c->dbg_bar_drop = drop_block;
    if (c->gexec) {   /* graphs hold the launch parameters they were captured with */
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    return MD_OK;
}

md_status md_set_graphs(md_ctx *c, int use_graphs)
{
    if (!c) return MD_ERR_ARG;
    c->use_graphs = use_graphs ? 1 : 0;
    return MD_OK;
}

md_status md_set_graph_rebuild(md_ctx *c, int inline_passes)
{
    if (!c) return MD_ERR_ARG;
    const int v = inline_passes ? 1 : 0;
    if (c->gexec && v != c->rebuild_inline) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    c->rebuild_inline = v;
    return MD_OK;
}

md_status md_set_fused_step(md_ctx *c, int fused)
{
    if (!c) return MD_ERR_ARG;
    const int old = c->fuse_step;
    c->fuse_step = 1;
    if (fused && !md_can_fuse(c)) {
        c->fuse_step = old;
        return fail(c, MD_ERR_UNSUPPORTED,
                    "md_set_fused_step: only leapfrog single systems without bonded terms fuse");
    }
    c->fuse_step = fused ? 1 : 0;
    if (c->gexec && c->fuse_step != old) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    return MD_OK;
}

md_status md_set_pair_depth(md_ctx *c, int depth)
{
    if (!c) return MD_ERR_ARG;
    const int t = c->pair_tpa;
    const int def = t >= 32 ? 1 : (t >= 16 ? 2 : (t >= 8 ? 4 : 8));
    if (depth == def) depth = 0;
    const bool ok = depth == 0 || (t == 4 && depth == 4) || (t == 8 && depth == 2) || (t == 16 && depth == 1);
    if (!ok) return fail(c, MD_ERR_ARG, "md_set_pair_depth: depth not built for this lane count");
    c->pair_depth = depth;
    if (c->gexec) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    return MD_OK;
}

md_status md_set_tuning(md_ctx *c, int pair_tpa, int list_tpa)
{
    if (!c) return MD_ERR_ARG;
    auto ok = [](int t) { return t == 1 || t == 2 || t == 4 || t == 8 || t == 16 || t == 32; };
    if (!ok(pair_tpa) || !(list_tpa == 0 || ok(list_tpa))) return MD_ERR_ARG;
    if (c->batch && list_tpa != 0)
        return fail(c, MD_ERR_ARG, "md_set_tuning: a batch builds its lists one warp per cell");
    c->pair_tpa = pair_tpa;
    c->pair_depth = 0;
    c->list_tpa = list_tpa;
    if (c->gexec) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    return MD_OK;
}

}  /* extern "C" */
