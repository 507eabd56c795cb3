/*
 * oracle.c -- CPU restatement of md_gpu's force-and-integrate path.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Built with -O2 -ffp-contract=off
 * so that every FP32 expression rounds exactly as written.  Each function
 * cites the reference lines it restates (paths relative to the md_gpu tree).
 */
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Constants with the values the reference stores (simulation.h:37-44,
 * forces.cu:47-55).  They are the Abramowitz & Stegun 7.1.26 coefficients and
 * the Coulomb factor e^2/(4 pi eps0) in kJ A/mol. */
#define ORC_PI_F   3.1415927f
#define ORC_A1     0.254829592f
#define ORC_A2     -0.284496736f
#define ORC_A3     1.421413741f
#define ORC_A4     -1.453152027f
#define ORC_A5     1.061405429f
#define ORC_PEX    0.3275911f
#define ORC_QFAC   1389.35427611722f
#define ORC_RGAS   8.314e-3   /* kJ/mol/K, as integrator.cu:155 (1000/8.314) */

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* input files                                                               */
/* ------------------------------------------------------------------------ */

/* simulation.cu:58-105.  Reads the positional .inp grammar; the label token
 * of each line is skipped.  Lines after rdel are extension lines of the form
 * "label value"; unknown labels are ignored. */
int orc_read_inp(const char *path, orc_params *p)
{
    FILE *fin = fopen(path, "r");
    if (!fin) return -1;
    char saux[256], ens[64];
    memset(p, 0, sizeof(*p));
    p->tau_t = 100.0f;
    if (fscanf(fin, "%255s %63s", saux, ens) != 2) { fclose(fin); return -2; }
    p->enstype = 0;
    if (strcmp(ens, "nvt") == 0) {
        p->enstype = 1;
        if (fscanf(fin, "%255s %f", saux, &p->temper_0) != 2) { fclose(fin); return -2; }
    }
    if (strcmp(ens, "npt") == 0) {
        p->enstype = 2;
        if (fscanf(fin, "%255s %f %f", saux, &p->temper_0, &p->press_0) != 3) { fclose(fin); return -2; }
    }
    if (fscanf(fin, "%255s %d %d %d %f", saux, &p->timeq, &p->timrun, &p->timprn, &p->dt) != 5) { fclose(fin); return -2; }
    if (fscanf(fin, "%255s %f %d", saux, &p->rcutsq, &p->lkspace) != 3) { fclose(fin); return -2; }
    if (p->lkspace == 0) {
        float eps;
        if (fscanf(fin, "%255s %f", saux, &eps) != 2) { fclose(fin); return -2; }
        /* float quotient, then divided by a double pow (simulation.cu:86) */
        float num = 2.0f * (eps - 1.0f) / (2.0f * eps + 1.0f);
        p->reacf = (float)((double)num / pow((double)p->rcutsq, 3.0));
    } else if (p->lkspace == 1) {
        if (fscanf(fin, "%255s %f", saux, &p->alfa) != 2) { fclose(fin); return -2; }
    } else {
        if (fscanf(fin, "%255s %d", saux, &p->kmax) != 2) { fclose(fin); return -2; }
        p->alfa = (float)(3.09 / (double)p->rcutsq);
    }
    p->rcutsq *= p->rcutsq;
    if (fscanf(fin, "%255s %f %d", saux, &p->skin, &p->nmaxlist) != 3) { fclose(fin); return -2; }
    if (fscanf(fin, "%255s %f", saux, &p->rdel) != 2) { fclose(fin); return -2; }
    /* extension lines */
    char val[64];
    while (fscanf(fin, "%255s %63s", saux, val) == 2) {
        if (strcmp(saux, "tau_t:") == 0) p->tau_t = strtof(val, NULL);
        else if (strcmp(saux, "integrator:") == 0) {
            if (strcmp(val, "vv") == 0) p->integrator = 1;
            else if (strcmp(val, "nh") == 0) p->integrator = 2;
            else p->integrator = 0;
        }
    }
    fclose(fin);
    return 0;
}

/* simulation.cu:144-264.  LJ tables use the reference's float/double mix:
 * lj1 = (float)((48 eps)_f * pow(sigma,12)), lj2 likewise with 24, pow 6. */
int orc_read_fld(const char *path, orc_ffield *f)
{
    FILE *fin = fopen(path, "r");
    if (!fin) return -1;
    char saux[256];
    int i, j, iaux, nvdw;
    float a, b;
    memset(f, 0, sizeof(*f));
    if (fscanf(fin, "%255s %d", saux, &f->ntype) != 2) goto bad;
    if (f->ntype < 1 || f->ntype > ORC_MAXTYPE) goto bad;
    for (int it = 0; it < f->ntype; it++) {
        if (fscanf(fin, "%d %d", &iaux, &f->nt[it]) != 2) goto bad;
        if (fscanf(fin, "%15s %f %f", f->name[it], &f->mass[it], &f->charge[it]) != 3) goto bad;
        f->mass[it] = (float)((double)f->mass[it] * 10000.0);
    }
    if (fscanf(fin, "%255s %d", saux, &nvdw) != 2) goto bad;
    for (int it = 0; it < nvdw; it++) {
        if (fscanf(fin, "%d %d %255s %f %f", &i, &j, saux, &a, &b) != 5) goto bad;
        i--; j--;
        if (i < 0 || j < 0 || i >= f->ntype || j >= f->ntype) goto bad;
        if (strcmp(saux, "LJ") == 0) {
            f->lj1[i * f->ntype + j] = (float)((double)(12.0f * 4.0f * b) * pow((double)a, 12.0));
            f->lj1[j * f->ntype + i] = f->lj1[i * f->ntype + j];
            f->lj2[i * f->ntype + j] = (float)((double)(6.0f * 4.0f * b) * pow((double)a, 6.0));
            f->lj2[j * f->ntype + i] = f->lj2[i * f->ntype + j];
        } else if (strcmp(saux, "12-6") == 0) {
            f->lj1[i * f->ntype + j] = 12.0f * a;
            f->lj1[j * f->ntype + i] = f->lj1[i * f->ntype + j];
            f->lj2[i * f->ntype + j] = 6.0f * b;
            f->lj2[j * f->ntype + i] = f->lj2[i * f->ntype + j];
        }
    }
    if (fscanf(fin, "%255s %d", saux, &f->tbonds) != 2) goto bad;
    if (f->tbonds < 0 || f->tbonds > ORC_MAXTYPE) goto bad;
    for (int it = 0; it < f->tbonds; it++) {
        if (fscanf(fin, "%d %f %f", &iaux, &f->bnd1[it], &f->bnd2[it]) != 3) goto bad;
        f->bnd1[it] *= 2.0f;
    }
    if (fscanf(fin, "%255s %d", saux, &f->tangle) != 2) goto bad;
    if (f->tangle < 0 || f->tangle > ORC_MAXTYPE) goto bad;
    for (int it = 0; it < f->tangle; it++) {
        if (fscanf(fin, "%d %f %f", &iaux, &f->ang1[it], &f->ang2[it]) != 3) goto bad;
        f->ang1[it] *= 2.0f;
        f->ang2[it] *= ORC_PI_F / 180.0f;
    }
    if (fscanf(fin, "%255s %d", saux, &f->nbonds) != 2) goto bad;
    f->bonds = (int *)malloc(sizeof(int) * 3 * (size_t)(f->nbonds > 0 ? f->nbonds : 1));
    for (int it = 0; it < f->nbonds; it++) {
        int *bd = f->bonds + 3 * it;
        if (fscanf(fin, "%d %d %d %d", &iaux, &bd[0], &bd[1], &bd[2]) != 4) goto bad;
    }
    if (fscanf(fin, "%255s %d", saux, &f->nangle) != 2) goto bad;
    f->angles = (int *)malloc(sizeof(int) * 4 * (size_t)(f->nangle > 0 ? f->nangle : 1));
    for (int it = 0; it < f->nangle; it++) {
        int *an = f->angles + 4 * it;
        if (fscanf(fin, "%d %d %d %d %d", &iaux, &an[0], &an[1], &an[2], &an[3]) != 5) goto bad;
    }
    fclose(fin);
    return 0;
bad:
    fclose(fin);
    return -2;
}

void orc_free_fld(orc_ffield *f)
{
    free(f->bonds); f->bonds = NULL;
    free(f->angles); f->angles = NULL;
}

/* simulation.cu:278-316.  boxi = 1.0/box in double, rounded to float. */
int orc_read_cfg(const char *path, const orc_ffield *f, orc_config *c)
{
    FILE *fin = fopen(path, "r");
    if (!fin) return -1;
    int iaux;
    memset(c, 0, sizeof(*c));
    if (fscanf(fin, "%d %d", &c->natom, &c->cftyp) != 2 || c->natom <= 0) { fclose(fin); return -2; }
    if (fscanf(fin, "%f %f %f", &c->box[0], &c->box[1], &c->box[2]) != 3) { fclose(fin); return -2; }
    for (int d = 0; d < 3; d++) c->boxi[d] = (float)(1.0 / (double)c->box[d]);
    size_t n = (size_t)c->natom;
    c->itype = (int *)calloc(n, sizeof(int));
    c->q = (float *)calloc(n, sizeof(float));
    c->pos = (float *)calloc(3 * n, sizeof(float));
    c->vel = (float *)calloc(3 * n, sizeof(float));
    c->mass = (float *)calloc(n, sizeof(float));
    for (size_t i = 0; i < n; i++) {
        if (fscanf(fin, "%d %d %f", &iaux, &c->itype[i], &c->q[i]) != 3) { fclose(fin); return -2; }
        c->itype[i] -= 1;
        if (c->itype[i] < 0 || c->itype[i] >= f->ntype) { fclose(fin); return -3; }
        c->mass[i] = f->mass[c->itype[i]];
        if (fscanf(fin, "%f %f %f", &c->pos[3 * i], &c->pos[3 * i + 1], &c->pos[3 * i + 2]) != 3) { fclose(fin); return -2; }
        if (c->cftyp > 0)
            if (fscanf(fin, "%f %f %f", &c->vel[3 * i], &c->vel[3 * i + 1], &c->vel[3 * i + 2]) != 3) { fclose(fin); return -2; }
    }
    fclose(fin);
    return 0;
}

void orc_free_cfg(orc_config *c)
{
    free(c->itype); free(c->q); free(c->pos); free(c->vel); free(c->mass);
    memset(c, 0, sizeof(*c));
}

/* simulation.cu:331-339 writes "%f"; this writer keeps that layout. */
int orc_write_cfg(const char *path, const orc_config *c, const float *pos3, const float *vel3)
{
    FILE *fo = fopen(path, "w");
    if (!fo) return -1;
    fprintf(fo, "%d %d\n", c->natom, 1);
    fprintf(fo, "%f %f %f\n", c->box[0], c->box[1], c->box[2]);
    for (int i = 0; i < c->natom; i++) {
        fprintf(fo, "%d %d %f\n", i + 1, c->itype[i] + 1, c->q[i]);
        fprintf(fo, "%f %f %f\n", pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2]);
        fprintf(fo, "%f %f %f\n", vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2]);
    }
    fclose(fo);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* packing and constants                                                     */
/* ------------------------------------------------------------------------ */

/* config.cu:34 */
void orc_pack_pos4(int n, const float *pos3, const int *itype, const float *q, float *pos4)
{
    for (int i = 0; i < n; i++) {
        pos4[4 * i + 0] = pos3[3 * i + 0];
        pos4[4 * i + 1] = pos3[3 * i + 1];
        pos4[4 * i + 2] = pos3[3 * i + 2];
        pos4[4 * i + 3] = (float)itype[i] + 0.1f * (q[i] + 5.0f);
    }
}

void orc_pack_vel4(int n, const float *vel3, const float *mass, float *vel4)
{
    for (int i = 0; i < n; i++) {
        vel4[4 * i + 0] = vel3[3 * i + 0];
        vel4[4 * i + 1] = vel3[3 * i + 1];
        vel4[4 * i + 2] = vel3[3 * i + 2];
        vel4[4 * i + 3] = mass[i];
    }
}

/* pair_forces.cu:44-45 */
float orc_decode_q(float w)
{
    int it = (int)floorf(w);
    return (w - (float)it) * 10.0f - 5.0f;
}

/* gpu_properties.cu:54 with block 256 */
int orc_pitch(int n) { return ((n + 255) / 256) * 256; }

/* neighborlist.cu:35.  The reference is C++: sqrt of a float is the float
 * overload, pow(float, int) promotes to double. */
float orc_rskinsq(float skin, float rcutsq)
{
    return (float)pow((double)(skin + sqrtf(rcutsq)), 2.0);
}

/* neighborlist.cu:36 */
float orc_rmaxdif(float skin) { return skin * skin / 4.0f; }

/* forces.cu:97-110: palfa, spiialfa, alfasq, wolf (wolf = 0 unless Wolf).
 * All float: in C++ sqrt of a float argument is the float overload. */
void orc_wolf_consts(float alfa, float rcutsq, float out4[4])
{
    float palfa = alfa * ORC_PEX;
    float spiialfa = 2.0f / sqrtf(ORC_PI_F) * alfa;
    float alfasq = -alfa * alfa / logf(2.0f);
    float ff = 1.0f / (1.0f + palfa * sqrtf(rcutsq));
    float wolf = spiialfa * sqrtf(rcutsq) + ((((ORC_A5 * ff + ORC_A4) * ff + ORC_A3) * ff + ORC_A2) * ff + ORC_A1) * ff;
    wolf *= exp2f(alfasq * rcutsq) / sqrtf(rcutsq);
    out4[0] = palfa; out4[1] = spiialfa; out4[2] = alfasq; out4[3] = wolf;
}

/* ------------------------------------------------------------------------ */
/* neighbour list                                                            */
/* ------------------------------------------------------------------------ */

/* neighborlist.cu:64-97, including its slot choice for the second atom (the
 * tests look at excl[i], not excl[j], when picking excl[j]'s slot).  Returns
 * the number of exclusions dropped because four slots were full. */
int orc_build_exclusions(int n, int nbonds, const int *bonds, unsigned *excl4)
{
    unsigned nat = (unsigned)n;
    int dropped = 0;
    for (int i = 0; i < 4 * n; i++) excl4[i] = nat + 1;
    for (int it = 0; it < nbonds; it++) {
        unsigned i = (unsigned)(bonds[3 * it + 1] - 1);
        unsigned j = (unsigned)(bonds[3 * it + 2] - 1);
        unsigned *ei = excl4 + 4 * i, *ej = excl4 + 4 * j;
        if (ei[0] > nat) ei[0] = j;
        else if (ei[1] > nat) ei[1] = j;
        else if (ei[2] > nat) ei[2] = j;
        else if (ei[3] > nat) ei[3] = j;
        else dropped++;
        if (ej[0] > nat) ej[0] = i;
        else if (ei[1] > nat) ej[1] = i;
        else if (ei[2] > nat) ej[2] = i;
        else if (ei[3] > nat) ej[3] = i;
        else dropped++;
    }
    return dropped;
}

/* The FP32 minimum-image squared distance exactly as neighborlist.cu:268-283
 * writes it, every operation rounded separately. */
static inline float mi_rsq_f32(float px, float py, float pz, const float *pj,
                               const float box[3], const float boxi[3])
{
    float dx = px - pj[0];
    float dy = py - pj[1];
    float dz = pz - pj[2];
    dx -= box[0] * rintf(dx * boxi[0]);
    dy -= box[1] * rintf(dy * boxi[1]);
    dz -= box[2] * rintf(dz * boxi[2]);
    return dx * dx + dy * dy + dz * dz;
}

/* neighborlist.cu:231-297: j ascending, r^2 < rskinsq, j != i, j not in the
 * four exclusion slots.  Entries beyond nmax are counted but not written.
 * Returns the largest per-atom count. */
int orc_nlist_nsquared(int n, const float *pos4, const float box[3], const float boxi[3],
                       float rskinsq, const unsigned *excl4, int pitch, int nmax,
                       unsigned *nnlist, unsigned *nnlist_max)
{
    int maxcount = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(max : maxcount)
    for (int i = 0; i < n; i++) {
        float px = pos4[4 * i], py = pos4[4 * i + 1], pz = pos4[4 * i + 2];
        const unsigned *ex = excl4 + 4 * i;
        int ibin = 0;
        for (int j = 0; j < n; j++) {
            float rsq = mi_rsq_f32(px, py, pz, pos4 + 4 * j, box, boxi);
            unsigned uj = (unsigned)j;
            if (rsq < rskinsq && j != i && uj != ex[0] && uj != ex[1] && uj != ex[2] && uj != ex[3]) {
                if (ibin < nmax) nnlist[i + (size_t)pitch * ibin] = uj;
                ibin++;
            }
        }
        nnlist_max[i] = (unsigned)ibin;
        if (ibin > maxcount) maxcount = ibin;
    }
    for (int i = n; i < pitch; i++) nnlist_max[i] = 0;
    return maxcount;
}

/* neighborlist.cu:157-176 */
int orc_nlist_check(int n, const float *pos4, const float *pos_old4, const float box[3],
                    const float boxi[3], float rmaxdif)
{
    int update = 0;
    for (int i = 0; i < n; i++) {
        float dx = pos4[4 * i] - pos_old4[4 * i];
        float dy = pos4[4 * i + 1] - pos_old4[4 * i + 1];
        float dz = pos4[4 * i + 2] - pos_old4[4 * i + 2];
        dx -= box[0] * rintf(dx * boxi[0]);
        dy -= box[1] * rintf(dy * boxi[1]);
        dz -= box[2] * rintf(dz * boxi[2]);
        if ((dx * dx + dy * dy + dz * dz) >= rmaxdif) update = 1;
    }
    return update;
}

/* ------------------------------------------------------------------------ */
/* cells and the Hilbert order                                               */
/* ------------------------------------------------------------------------ */

/* Cells of side >= rl/2 (with a 1e-4 margin), at least one per axis. */
void orc_cell_dims(const float box[3], float rl, int ncell[3], float binlen[3])
{
    for (int d = 0; d < 3; d++) {
        int nc = (int)floorf(box[d] / (0.5f * rl * 1.0001f));
        if (nc < 1) nc = 1;
        if (nc > 1024) nc = 1024;
        ncell[d] = nc;
        binlen[d] = box[d] / (float)nc;
    }
}

/* Cell of a centred coordinate, the binning rule the reference sketches in
 * neighborlist_kernel_o.cu:20-25 ((x + L/2) / bin, truncated), clamped to the
 * grid so that x = +L/2 (reachable after the wrap in nve_leapfrog.cu:52) stays
 * inside. */
static inline int cell_of(float x, float box, float binlen, int nc)
{
    float s = (x + box / 2.0f) / binlen;
    int c = (s <= 0.0f) ? 0 : (int)s;
    if (c >= nc) c = nc - 1;
    return c;
}

void orc_cell_index(int n, const float *pos4, const float box[3], const int ncell[3],
                    const float binlen[3], int *cell3)
{
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++)
            cell3[3 * i + d] = cell_of(pos4[4 * i + d], box[d], binlen[d], ncell[d]);
}

/* 3-D Hilbert index of a point on a 2^bits grid: J. Skilling, "Programming
 * the Hilbert curve", AIP Conf. Proc. 707 (2004) 381 (axes -> transpose,
 * then bit interleave). */
unsigned long long orc_hilbert3(unsigned x, unsigned y, unsigned z, int bits)
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
        for (int i = 0; i < 3; i++)
            h = (h << 1) | ((X[i] >> b) & 1u);
    return h;
}

/* ------------------------------------------------------------------------ */
/* pair forces                                                               */
/* ------------------------------------------------------------------------ */

/* pair_forces.cu:34-131 (kind 0, reaction field) and :133-205 (kind 1,
 * LJ + Wolf), FP32 as written.  wc = orc_wolf_consts() output. */
void orc_pair_f32(int kind, int n, const float *pos4, const float box[3], const float boxi[3],
                  const unsigned *nnlist, const unsigned *nnlist_max, int pitch, int ntype,
                  const float *lj1, const float *lj2, float rcutsq, float reacf,
                  const float wc[4], float *force4)
{
    const float palfa = wc[0], spiialfa = wc[1], alfasq = wc[2], wolf = wc[3];
    const float qfac = ORC_QFAC;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        const float *pi = pos4 + 4 * i;
        int num = (int)nnlist_max[i];
        int it = (int)floorf(pi[3]);
        float qi = (pi[3] - (float)it) * 10.0f - 5.0f;
        it *= ntype;
        float fx = 0.0f, fy = 0.0f, fz = 0.0f, fw = 0.0f;
        for (int jx = 0; jx < num; jx++) {
            unsigned j = nnlist[i + (size_t)pitch * jx];
            const float *pj = pos4 + 4 * (size_t)j;
            int jt = (int)floorf(pj[3]);
            float qj = (pj[3] - (float)jt) * 10.0f - 5.0f;
            jt += it;
            float lja = lj1[jt], ljc = lj2[jt];
            float dx = pi[0] - pj[0];
            float dy = pi[1] - pj[1];
            float dz = pi[2] - pj[2];
            dx -= box[0] * rintf(dx * boxi[0]);
            dy -= box[1] * rintf(dy * boxi[1]);
            dz -= box[2] * rintf(dz * boxi[2]);
            float rsq = dx * dx + dy * dy + dz * dz;
            float ri = 1.0f / sqrtf(rsq);
            float ff;
            if (kind == 0) {
                ff = qfac * qi * qj * (ri - reacf * rsq);
            } else {
                ff = 1.0f / (1.0f + palfa * rsq * ri);
                ff = spiialfa * rsq * ri + ((((ORC_A5 * ff + ORC_A4) * ff + ORC_A3) * ff + ORC_A2) * ff + ORC_A1) * ff;
                ff *= exp2f(alfasq * rsq) * ri;
                ff -= wolf;
                ff *= qfac * qi * qj;
            }
            ri *= ri;
            ff *= ri;
            ri *= ri; ri *= ri;
            ff += (lja * ri * rsq - ljc) * ri;
            if (rsq > rcutsq) ff = 0.0f;
            fw += ff * rsq;
            fx += ff * dx;
            fy += ff * dy;
            fz += ff * dz;
        }
        force4[4 * i + 0] = fx; force4[4 * i + 1] = fy;
        force4[4 * i + 2] = fz; force4[4 * i + 3] = fw;
    }
}

/* erfc by A&S 7.1.26 with the reference's float coefficients, in FP64. */
static inline double erfc_as(double x)
{
    double t = 1.0 / (1.0 + (double)ORC_PEX * x);
    double p = ((((double)ORC_A5 * t + (double)ORC_A4) * t + (double)ORC_A3) * t + (double)ORC_A2) * t + (double)ORC_A1;
    return p * t * exp(-x * x);
}

typedef struct {
    int kind, erfc_exact;
    double rc, rcsq, reacf, alpha, spi, wolfW, ucoul_c;
} pairmodel;

static void pairmodel_init(pairmodel *m, int kind, int erfc_exact, float rcutsq, float reacf, float alfa)
{
    m->kind = kind;
    m->erfc_exact = erfc_exact;
    m->rcsq = (double)rcutsq;
    m->rc = sqrt(m->rcsq);
    m->reacf = (double)reacf;
    m->alpha = (double)alfa;
    m->spi = 2.0 / sqrt(3.14159265358979323846) * m->alpha;
    if (kind == 1) {
        double ec = erfc_exact ? erfc(m->alpha * m->rc) : erfc_as(m->alpha * m->rc);
        /* W = rc * Ft(rc), Ft(r) = erfc(a r)/r^2 + 2a/sqrt(pi) exp(-a^2 r^2)/r (forces.cu:104-110) */
        m->wolfW = ec / m->rc + m->spi * exp(-m->alpha * m->alpha * m->rcsq);
        m->ucoul_c = ec / m->rc;
    } else {
        m->wolfW = 0.0;
        m->ucoul_c = 1.0 / m->rc + 0.5 * m->reacf * m->rcsq;
    }
}

/* Pair force factor ff (F_vec = ff * d) and pair energy for r^2 <= rc^2. */
static inline void pair_eval_f64(const pairmodel *m, double rsq, double qq, double lja, double ljc,
                                 double *ff_out, double *u_out)
{
    double r = sqrt(rsq), ri = 1.0 / r, ri2 = ri * ri;
    double fc, uc;
    if (m->kind == 0) {
        fc = qq * (ri * ri2 - m->reacf);
        uc = qq * (ri + 0.5 * m->reacf * rsq - m->ucoul_c);
    } else {
        double x = m->alpha * r;
        double ec = m->erfc_exact ? erfc(x) : erfc_as(x);
        double g = ec * ri + m->spi * exp(-x * x);
        fc = qq * (g - m->wolfW) * ri2;
        uc = qq * (ec * ri - m->ucoul_c + m->wolfW * log(r / m->rc));
    }
    double ri6 = ri2 * ri2 * ri2, ri8 = ri6 * ri2;
    double rc2i = 1.0 / m->rcsq, rc6i = rc2i * rc2i * rc2i;
    double flj = lja * ri6 * ri8 - ljc * ri8;
    double ulj = lja / 12.0 * (ri6 * ri6 - rc6i * rc6i) - ljc / 6.0 * (ri6 - rc6i);
    *ff_out = fc + flj;
    *u_out = uc + ulj;
}

/* FP64 plain form of the pair forces over a given list: positions as stored,
 * charges as read (not decoded from w), the model constants above.  force4 =
 * (fx, fy, fz, sum ff r^2) like the reference; epot[i] = half of the pair
 * energies of i (consistent potential, shifted LJ). */
void orc_pair_f64(int kind, int erfc_exact, int n, const float *pos4, const int *itype,
                  const float *q, const float box[3], const unsigned *nnlist,
                  const unsigned *nnlist_max, int pitch, int ntype, const float *lj1,
                  const float *lj2, float rcutsq, float reacf, float alfa,
                  double *force4, double *epot)
{
    pairmodel m;
    pairmodel_init(&m, kind, erfc_exact, rcutsq, reacf, alfa);
    const double qfac = (double)ORC_QFAC;
    const double L[3] = {box[0], box[1], box[2]};
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < n; i++) {
        double fx = 0, fy = 0, fz = 0, fw = 0, u = 0;
        double xi = pos4[4 * i], yi = pos4[4 * i + 1], zi = pos4[4 * i + 2];
        int num = (int)nnlist_max[i];
        for (int jx = 0; jx < num; jx++) {
            unsigned j = nnlist[i + (size_t)pitch * jx];
            double dx = xi - (double)pos4[4 * j], dy = yi - (double)pos4[4 * j + 1], dz = zi - (double)pos4[4 * j + 2];
            dx -= L[0] * rint(dx / L[0]);
            dy -= L[1] * rint(dy / L[1]);
            dz -= L[2] * rint(dz / L[2]);
            double rsq = dx * dx + dy * dy + dz * dz;
            if (rsq > m.rcsq) continue;
            int t = itype[i] * ntype + itype[j];
            double ff, uu;
            pair_eval_f64(&m, rsq, qfac * (double)q[i] * (double)q[j], lj1[t], lj2[t], &ff, &uu);
            fx += ff * dx; fy += ff * dy; fz += ff * dz; fw += ff * rsq;
            u += 0.5 * uu;
        }
        force4[4 * i] = fx; force4[4 * i + 1] = fy; force4[4 * i + 2] = fz; force4[4 * i + 3] = fw;
        if (epot) epot[i] = u;
    }
}

static inline int is_excluded(const unsigned *excl4, int i, int j)
{
    if (!excl4) return 0;
    const unsigned *e = excl4 + 4 * i;
    unsigned uj = (unsigned)j;
    return uj == e[0] || uj == e[1] || uj == e[2] || uj == e[3];
}

/* List-free FP64 pair forces over all j != i inside rc (small systems). */
void orc_pair_allpairs_f64(int kind, int erfc_exact, int n, const float *pos4, const int *itype,
                           const float *q, const float box[3], int ntype, const float *lj1,
                           const float *lj2, float rcutsq, float reacf, float alfa,
                           const unsigned *excl4, double *force4, double *epot)
{
    pairmodel m;
    pairmodel_init(&m, kind, erfc_exact, rcutsq, reacf, alfa);
    const double qfac = (double)ORC_QFAC;
    const double L[3] = {box[0], box[1], box[2]};
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; i++) {
        double fx = 0, fy = 0, fz = 0, fw = 0, u = 0;
        double xi = pos4[4 * i], yi = pos4[4 * i + 1], zi = pos4[4 * i + 2];
        for (int j = 0; j < n; j++) {
            if (j == i || is_excluded(excl4, i, j)) continue;
            double dx = xi - (double)pos4[4 * j], dy = yi - (double)pos4[4 * j + 1], dz = zi - (double)pos4[4 * j + 2];
            dx -= L[0] * rint(dx / L[0]);
            dy -= L[1] * rint(dy / L[1]);
            dz -= L[2] * rint(dz / L[2]);
            double rsq = dx * dx + dy * dy + dz * dz;
            if (rsq > m.rcsq) continue;
            int t = itype[i] * ntype + itype[j];
            double ff, uu;
            pair_eval_f64(&m, rsq, qfac * (double)q[i] * (double)q[j], lj1[t], lj2[t], &ff, &uu);
            fx += ff * dx; fy += ff * dy; fz += ff * dz; fw += ff * rsq;
            u += 0.5 * uu;
        }
        force4[4 * i] = fx; force4[4 * i + 1] = fy; force4[4 * i + 2] = fz; force4[4 * i + 3] = fw;
        if (epot) epot[i] = u;
    }
}

/* Unordered pairs with r^2 < rc^2 (FP64 distances), exclusions removed. */
long long orc_count_pairs(int n, const float *pos4, const float box[3], float rcutsq,
                          const unsigned *excl4)
{
    long long cnt = 0;
    const double L[3] = {box[0], box[1], box[2]};
    const double rcsq = rcutsq;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : cnt)
    for (int i = 0; i < n; i++) {
        double xi = pos4[4 * i], yi = pos4[4 * i + 1], zi = pos4[4 * i + 2];
        for (int j = i + 1; j < n; j++) {
            double dx = xi - (double)pos4[4 * j], dy = yi - (double)pos4[4 * j + 1], dz = zi - (double)pos4[4 * j + 2];
            dx -= L[0] * rint(dx / L[0]);
            dy -= L[1] * rint(dy / L[1]);
            dz -= L[2] * rint(dz / L[2]);
            if (dx * dx + dy * dy + dz * dz < rcsq && !is_excluded(excl4, i, j)) cnt++;
        }
    }
    return cnt;
}

/* ------------------------------------------------------------------------ */
/* bonded forces                                                             */
/* ------------------------------------------------------------------------ */

/* forces.cu:118-134.  Returns -1 if an atom has more than four bonds (the
 * reference writes past its list then). */
int orc_bond_lists(int n, int nbonds, const int *bonds, int pitch, unsigned *bndlist2,
                   unsigned *bndlist_max)
{
    for (int i = 0; i < pitch; i++) bndlist_max[i] = 0;
    for (int it = 0; it < nbonds; it++) {
        unsigned i = (unsigned)(bonds[3 * it + 1] - 1), j = (unsigned)(bonds[3 * it + 2] - 1);
        unsigned t = (unsigned)(bonds[3 * it + 0] - 1);
        if (bndlist_max[i] >= 4 || bndlist_max[j] >= 4) return -1;
        size_t si = i + (size_t)bndlist_max[i] * pitch, sj = j + (size_t)bndlist_max[j] * pitch;
        bndlist2[2 * si] = j; bndlist2[2 * si + 1] = t;
        bndlist2[2 * sj] = i; bndlist2[2 * sj + 1] = t;
        bndlist_max[i]++; bndlist_max[j]++;
    }
    (void)n;
    return 0;
}

/* forces.cu:147-173: role 0 for the ends, 1 for the centre. */
int orc_angle_lists(int n, int nangle, const int *angles, int pitch, unsigned *anglist4,
                    unsigned *anglist_max)
{
    for (int i = 0; i < pitch; i++) anglist_max[i] = 0;
    for (int it = 0; it < nangle; it++) {
        unsigned t = (unsigned)(angles[4 * it] - 1);
        unsigned i = (unsigned)(angles[4 * it + 1] - 1), j = (unsigned)(angles[4 * it + 2] - 1),
                 k = (unsigned)(angles[4 * it + 3] - 1);
        if (anglist_max[i] >= 4 || anglist_max[j] >= 4 || anglist_max[k] >= 4) return -1;
        unsigned *e;
        e = anglist4 + 4 * (i + (size_t)anglist_max[i] * pitch); e[0] = 0; e[1] = j; e[2] = k; e[3] = t;
        e = anglist4 + 4 * (j + (size_t)anglist_max[j] * pitch); e[0] = 1; e[1] = i; e[2] = k; e[3] = t;
        e = anglist4 + 4 * (k + (size_t)anglist_max[k] * pitch); e[0] = 0; e[1] = j; e[2] = i; e[3] = t;
        anglist_max[i]++; anglist_max[j]++; anglist_max[k]++;
    }
    (void)n;
    return 0;
}

/* bonded_forces.cu:34-95, FP32 as written; adds into force4. */
void orc_bonds_f32(int n, const float *pos4, const float box[3], const float boxi[3],
                   const unsigned *bndlist2, const unsigned *bndlist_max, int pitch,
                   const float *bnd1, const float *bnd2, float *force4)
{
    for (int i = 0; i < n; i++) {
        const float *pi = pos4 + 4 * i;
        float *f = force4 + 4 * i;
        float fx = f[0], fy = f[1], fz = f[2], fw = f[3];
        int num = (int)bndlist_max[i];
        for (int jx = 0; jx < num; jx++) {
            size_t s = i + (size_t)pitch * jx;
            unsigned j = bndlist2[2 * s], jt = bndlist2[2 * s + 1];
            const float *pj = pos4 + 4 * (size_t)j;
            float kk = bnd1[jt], r0 = bnd2[jt];
            float dx = pi[0] - pj[0], dy = pi[1] - pj[1], dz = pi[2] - pj[2];
            dx -= box[0] * rintf(dx * boxi[0]);
            dy -= box[1] * rintf(dy * boxi[1]);
            dz -= box[2] * rintf(dz * boxi[2]);
            float rsq = dx * dx + dy * dy + dz * dz;
            float fa = kk * (r0 * (1.0f / sqrtf(rsq)) - 1.0f);
            fw += fa * rsq;
            fx += fa * dx; fy += fa * dy; fz += fa * dz;
        }
        f[0] = fx; f[1] = fy; f[2] = fz; f[3] = fw;
    }
}

/* bonded_forces.cu:98-193, FP32 as written; adds into force4.  The centre
 * branch at :173 tests the role of the entry already prefetched at :131-132,
 * i.e. of the next entry when there is one; this restatement keeps that. */
void orc_angles_f32(int n, const float *pos4, const float box[3], const float boxi[3],
                    const unsigned *anglist4, const unsigned *anglist_max, int pitch,
                    const float *ang1, const float *ang2, float *force4)
{
    for (int id = 0; id < n; id++) {
        const float *pd = pos4 + 4 * id;
        float *f = force4 + 4 * id;
        float fx = f[0], fy = f[1], fz = f[2];
        int num = (int)anglist_max[id];
        unsigned nj[4];
        memcpy(nj, anglist4 + 4 * (size_t)id, sizeof(nj));
        for (int jx = 0; jx < num; jx++) {
            const float *pj_ = pos4 + 4 * (size_t)nj[1];
            const float *pk = pos4 + 4 * (size_t)nj[2];
            float pi[3] = {pd[0], pd[1], pd[2]};
            float pj[3] = {pj_[0], pj_[1], pj_[2]};
            if (nj[0] == 1) {
                pi[0] = pj_[0]; pi[1] = pj_[1]; pi[2] = pj_[2];
                pj[0] = pd[0]; pj[1] = pd[1]; pj[2] = pd[2];
            }
            float ff = ang1[nj[3]], thet0 = ang2[nj[3]];
            if (jx < num - 1) memcpy(nj, anglist4 + 4 * (id + (size_t)(jx + 1) * pitch), sizeof(nj));
            float ax = pi[0] - pj[0], ay = pi[1] - pj[1], az = pi[2] - pj[2];
            ax -= box[0] * rintf(ax * boxi[0]);
            ay -= box[1] * rintf(ay * boxi[1]);
            az -= box[2] * rintf(az * boxi[2]);
            float ai = 1.0f / sqrtf(ax * ax + ay * ay + az * az);
            float bx = pk[0] - pj[0], by = pk[1] - pj[1], bz = pk[2] - pj[2];
            bx -= box[0] * rintf(bx * boxi[0]);
            by -= box[1] * rintf(by * boxi[1]);
            bz -= box[2] * rintf(bz * boxi[2]);
            float bi = 1.0f / sqrtf(bx * bx + by * by + bz * bz);
            float ab = ax * bx + ay * by + az * bz;
            float cang = ab * ai * bi;
            if (cang <= -0.9999999f) cang = -0.9999999f;
            if (cang >= 0.9999999f) cang = 0.9999999f;
            ff *= (acosf(cang) - thet0) * (1.0f / sqrtf(1.0f - cang * cang)) * ai * bi;
            ai = ab * ai * ai;
            float qx = bx - ai * ax, qy = by - ai * ay, qz = bz - ai * az;
            if (nj[0] == 1) {
                bi = ab * bi * bi;
                qx = bi * bx - ax - qx;
                qy = bi * by - ay - qy;
                qz = bi * bz - az - qz;
            }
            fx += ff * qx; fy += ff * qy; fz += ff * qz;
        }
        f[0] = fx; f[1] = fy; f[2] = fz;
    }
}

static inline void mi_d64(const float *a, const float *b, const double L[3], double d[3])
{
    for (int k = 0; k < 3; k++) {
        d[k] = (double)a[k] - (double)b[k];
        d[k] -= L[k] * rint(d[k] / L[k]);
    }
}

/* FP64 harmonic bonds U = k (r - r0)^2 with bnd1 = 2k, per bond; adds into
 * force4 and epot (the per-atom virial column gets fa r^2 for both atoms, as
 * the reference's per-atom lists do). */
void orc_bonds_f64(int n, const float *pos4, const float box[3], int nbonds, const int *bonds,
                   const float *bnd1, const float *bnd2, double *force4, double *epot)
{
    const double L[3] = {box[0], box[1], box[2]};
    for (int it = 0; it < nbonds; it++) {
        int t = bonds[3 * it] - 1, i = bonds[3 * it + 1] - 1, j = bonds[3 * it + 2] - 1;
        double d[3];
        mi_d64(pos4 + 4 * i, pos4 + 4 * j, L, d);
        double rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2], r = sqrt(rsq);
        double fa = (double)bnd1[t] * ((double)bnd2[t] / r - 1.0);
        for (int k = 0; k < 3; k++) { force4[4 * i + k] += fa * d[k]; force4[4 * j + k] -= fa * d[k]; }
        force4[4 * i + 3] += fa * rsq; force4[4 * j + 3] += fa * rsq;
        if (epot) {
            double u = 0.5 * (double)bnd1[t] * (r - bnd2[t]) * (r - bnd2[t]);
            epot[i] += 0.5 * u; epot[j] += 0.5 * u;
        }
    }
    (void)n;
}

/* FP64 harmonic angles U = k (theta - theta0)^2 with ang1 = 2k, per angle,
 * cos clamped to +-0.9999999 like bonded_forces.cu:154-155. */
void orc_angles_f64(int n, const float *pos4, const float box[3], int nangle, const int *angles,
                    const float *ang1, const float *ang2, double *force4, double *epot)
{
    const double L[3] = {box[0], box[1], box[2]};
    for (int it = 0; it < nangle; it++) {
        int t = angles[4 * it] - 1, i = angles[4 * it + 1] - 1, j = angles[4 * it + 2] - 1,
            k = angles[4 * it + 3] - 1;
        double a[3], b[3];
        mi_d64(pos4 + 4 * i, pos4 + 4 * j, L, a);
        mi_d64(pos4 + 4 * k, pos4 + 4 * j, L, b);
        double aa = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
        double bb = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
        double ab = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
        double ai = 1.0 / sqrt(aa), bi = 1.0 / sqrt(bb);
        double c = ab * ai * bi;
        if (c <= -0.9999999) c = -0.9999999;
        if (c >= 0.9999999) c = 0.9999999;
        double th = acos(c);
        double ff = (double)ang1[t] * (th - (double)ang2[t]) / sqrt(1.0 - c * c) * ai * bi;
        for (int d = 0; d < 3; d++) {
            double fi = ff * (b[d] - ab / aa * a[d]);
            double fk = ff * (a[d] - ab / bb * b[d]);
            force4[4 * i + d] += fi;
            force4[4 * k + d] += fk;
            force4[4 * j + d] -= fi + fk;
        }
        if (epot) {
            double u = 0.5 * (double)ang1[t] * (th - ang2[t]) * (th - ang2[t]);
            epot[i] += u / 3.0; epot[j] += u / 3.0; epot[k] += u / 3.0;
        }
    }
    (void)n;
}

/* ------------------------------------------------------------------------ */
/* integrators, as written                                                   */
/* ------------------------------------------------------------------------ */

/* nve_leapfrog.cu:31-60 */
void orc_leapfrog_nve_f32(int n, float *pos4, float *vel4, const float *force4, float dt,
                          const float box[3], const float boxi[3])
{
    for (int i = 0; i < n; i++) {
        float *v = vel4 + 4 * i, *x = pos4 + 4 * i;
        const float *f = force4 + 4 * i;
        float massif = dt / v[3];
        v[0] += f[0] * massif;
        v[1] += f[1] * massif;
        v[2] += f[2] * massif;
        for (int d = 0; d < 3; d++) {
            x[d] += v[d] * dt;
            x[d] -= box[d] * truncf(x[d] * 2.0f * boxi[d]);
        }
    }
}

/* nvt_leapfrog_ber.cu:29-80, with the per-block tree reduction of m v^2. */
void orc_leapfrog_nvt_f32(int n, float *pos4, float *vel4, const float *force4, float dt,
                          float scale, const float box[3], const float boxi[3], int block,
                          float *ke_partials)
{
    int nblocks = (n + block - 1) / block;
    float *sh = (float *)malloc(sizeof(float) * (size_t)block);
    for (int b = 0; b < nblocks; b++) {
        for (int t = 0; t < block; t++) {
            int i = b * block + t;
            if (i < n) {
                float *v = vel4 + 4 * i, *x = pos4 + 4 * i;
                const float *f = force4 + 4 * i;
                float massif = dt / v[3];
                v[0] = (v[0] + f[0] * massif) * scale;
                v[1] = (v[1] + f[1] * massif) * scale;
                v[2] = (v[2] + f[2] * massif) * scale;
                sh[t] = v[3] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                x[0] += v[0] * dt;
                x[1] += v[1] * dt;
                x[2] += v[2] * dt;
                for (int d = 0; d < 3; d++) x[d] -= box[d] * truncf(x[d] * 2.0f * boxi[d]);
            } else {
                sh[t] = 0.0f;
            }
        }
        for (int s = block >> 1; s > 0; s >>= 1)
            for (int t = 0; t < s; t++) sh[t] += sh[t + s];
        ke_partials[b] = sh[0];
    }
    free(sh);
}

/* nvt_leapfrog_ber.cu:83-110 launched with one block of nblocks threads
 * (integrator.cu:54-56): a tree over a non-power-of-two width drops terms. */
float orc_ke_sum_ref(int nblocks, const float *partials)
{
    int bd = nblocks;
    float *sh = (float *)malloc(sizeof(float) * (size_t)(bd > 0 ? bd : 1));
    float ksum = 0.0f;
    for (int ib = 0; ib < nblocks; ib += bd) {
        for (int t = 0; t < bd; t++) sh[t] = (ib + t < nblocks) ? partials[t + ib] : 0.0f;
        for (int s = bd >> 1; s > 0; s >>= 1)
            for (int t = 0; t < s; t++) sh[t] += sh[t + s];
        ksum += sh[0];
    }
    free(sh);
    return ksum;
}

/* integrator.cu:146-147 (tco = 0.01 as a float) */
float orc_berendsen_scale(float dt, float tco, float temper_0, float temper)
{
    return sqrtf(1.0f + dt * tco * (temper_0 / temper - 1.0f));
}

/* integrator.cu:154-155 */
float orc_temperature_ref(float ke_sum0, int n)
{
    float ke = ke_sum0 * 0.5f;
    float t = ke * 2.0f / (3.0f * (float)n - 3.0f);
    return (float)((double)t * 1000.0 / 8.314);
}

/* nve_vverlet.cu:31-58 as written (the drift adds the half kick twice). */
void orc_vv_pre_f32(int n, float *pos4, float *vel4, const float *force4, float dt,
                    const float box[3], const float boxi[3])
{
    float hdt = (float)(0.5 * (double)dt);
    for (int i = 0; i < n; i++) {
        float *v = vel4 + 4 * i, *x = pos4 + 4 * i;
        const float *f = force4 + 4 * i;
        float massif = hdt / v[3];
        v[0] += f[0] * massif;
        v[1] += f[1] * massif;
        v[2] += f[2] * massif;
        for (int d = 0; d < 3; d++) {
            x[d] += (v[d] + f[d] * massif) * dt;
            x[d] -= box[d] * truncf(x[d] * 2.0f * boxi[d]);
        }
    }
}

/* nve_vverlet.cu:61-79 */
void orc_vv_cor_f32(int n, float *vel4, const float *force4, float dt)
{
    float hdt = (float)(0.5 * (double)dt);
    for (int i = 0; i < n; i++) {
        float *v = vel4 + 4 * i;
        const float *f = force4 + 4 * i;
        float massif = hdt / v[3];
        v[0] += f[0] * massif;
        v[1] += f[1] * massif;
        v[2] += f[2] * massif;
    }
}

/* ------------------------------------------------------------------------ */
/* integrators, plain FP64                                                   */
/* ------------------------------------------------------------------------ */

void orc_wrap_f64(int n, double *x, const float box[3])
{
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            double L = box[d];
            x[3 * i + d] -= L * trunc(x[3 * i + d] * 2.0 / L);
        }
}

/* sum 1/2 m' v^2 in kJ/mol (m' = m * 1e4, v in A/fs) */
double orc_kinetic_f64(int n, const double *v, const double *m)
{
    double ke = 0.0;
    for (int i = 0; i < n; i++)
        ke += 0.5 * m[i] * (v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2]);
    return ke;
}

/* leapfrog with optional Berendsen scale (scale = 1 for NVE) */
void orc_leapfrog_f64(int n, double *x, double *v, const double *f, const double *m,
                      double dt, double scale, const float box[3])
{
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            v[3 * i + d] = (v[3 * i + d] + f[3 * i + d] * dt / m[i]) * scale;
            x[3 * i + d] += v[3 * i + d] * dt;
        }
    orc_wrap_f64(n, x, box);
}

void orc_vv_kick_f64(int n, double *v, const double *f, const double *m, double half_dt)
{
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) v[3 * i + d] += f[3 * i + d] * half_dt / m[i];
}

void orc_vv_drift_f64(int n, double *x, const double *v, double dt, const float box[3])
{
    for (int i = 0; i < 3 * n; i++) x[i] += v[i] * dt;
    orc_wrap_f64(n, x, box);
}

/* Half step of a single Nose-Hoover thermostat (Martyna-Klein-Tuckerman,
 * Trotter splitting, e.g. Frenkel & Smit 2nd ed. Alg. 30 with one chain
 * element): xi += G dt/4; v *= exp(-xi dt/2); eta += xi dt/2; xi += G dt/4,
 * G = (2K - ndf kT0)/Q. */
void orc_nh_half_f64(int n, double *v, const double *m, double dt, double t0, double q_nh,
                     int ndf, double *xi, double *eta)
{
    double kt = ORC_RGAS * t0;
    double ke = orc_kinetic_f64(n, v, m);
    *xi += 0.25 * dt * (2.0 * ke - ndf * kt) / q_nh;
    double s = exp(-0.5 * dt * (*xi));
    for (int i = 0; i < 3 * n; i++) v[i] *= s;
    ke *= s * s;
    *eta += 0.5 * dt * (*xi);
    *xi += 0.25 * dt * (2.0 * ke - ndf * kt) / q_nh;
}

/* ------------------------------------------------------------------------ */
/* whole runs                                                                */
/* ------------------------------------------------------------------------ */

int orc_md_ref_run(const orc_params *p, const orc_ffield *f, int n, float *pos4, float *vel4,
                   const float box[3], const float boxi[3], int nsteps, int exact_ke,
                   float *force4_out, float *temper_io, float *temps_out)
{
    int have = 0;
    return orc_md_ref_run_cont(p, f, n, pos4, vel4, box, boxi, nsteps, exact_ke, NULL, NULL, NULL, &have,
                               force4_out, temper_io, temps_out);
}

int orc_md_ref_run_cont(const orc_params *p, const orc_ffield *f, int n, float *pos4, float *vel4,
                        const float box[3], const float boxi[3], int nsteps, int exact_ke,
                        unsigned *nnl_io, unsigned *nnm_io, float *pold_io, int *have_list,
                        float *force4_out, float *temper_io, float *temps_out)
{
    int pitch = orc_pitch(n), nmax = p->nmaxlist;
    int kind = p->lkspace == 0 ? 0 : 1;
    float rskinsq = orc_rskinsq(p->skin, p->rcutsq), rmaxdif = orc_rmaxdif(p->skin);
    float wc[4] = {0, 0, 0, 0};
    if (p->lkspace > 0) orc_wolf_consts(p->alfa, p->rcutsq, wc);
    if (p->lkspace != 1) wc[3] = 0.0f;
    unsigned *excl = (unsigned *)malloc(sizeof(unsigned) * 4 * (size_t)n);
    const int own = nnl_io == NULL;
    unsigned *nnl = own ? (unsigned *)malloc(sizeof(unsigned) * (size_t)pitch * (size_t)nmax) : nnl_io;
    unsigned *nnm = own ? (unsigned *)malloc(sizeof(unsigned) * (size_t)pitch) : nnm_io;
    float *pold = own ? (float *)malloc(sizeof(float) * 4 * (size_t)n) : pold_io;
    float *frc = (float *)malloc(sizeof(float) * 4 * (size_t)n);
    int nblk = (n + 255) / 256;
    float *part = (float *)malloc(sizeof(float) * (size_t)nblk);
    unsigned *bl = NULL, *blm = NULL, *al = NULL, *alm = NULL;
    int rc = 0, builds = 0;
    orc_build_exclusions(n, f->nbonds, f->bonds, excl);
    if (f->nbonds > 0) {
        bl = (unsigned *)calloc((size_t)pitch * 4 * 2, sizeof(unsigned));
        blm = (unsigned *)calloc((size_t)pitch, sizeof(unsigned));
        if (orc_bond_lists(n, f->nbonds, f->bonds, pitch, bl, blm)) { rc = -2; goto done; }
    }
    if (f->nangle > 0) {
        al = (unsigned *)calloc((size_t)pitch * 4 * 4, sizeof(unsigned));
        alm = (unsigned *)calloc((size_t)pitch, sizeof(unsigned));
        if (orc_angle_lists(n, f->nangle, f->angles, pitch, al, alm)) { rc = -2; goto done; }
    }
    float temper = temper_io ? *temper_io : p->temper_0;
    if (!*have_list) {   /* neighborlist_init: the first build */
        if (orc_nlist_nsquared(n, pos4, box, boxi, rskinsq, excl, pitch, nmax, nnl, nnm) > nmax) { rc = -1; goto done; }
        memcpy(pold, pos4, sizeof(float) * 4 * (size_t)n);
        builds = 1;
        *have_list = 1;
    }
    for (int t = 0; t < nsteps; t++) {
        if (orc_nlist_check(n, pos4, pold, box, boxi, rmaxdif)) {
            if (orc_nlist_nsquared(n, pos4, box, boxi, rskinsq, excl, pitch, nmax, nnl, nnm) > nmax) { rc = -1; goto done; }
            memcpy(pold, pos4, sizeof(float) * 4 * (size_t)n);
            builds++;
        }
        orc_pair_f32(kind, n, pos4, box, boxi, nnl, nnm, pitch, f->ntype, f->lj1, f->lj2, p->rcutsq, p->reacf, wc, frc);
        if (f->nbonds > 0) orc_bonds_f32(n, pos4, box, boxi, bl, blm, pitch, f->bnd1, f->bnd2, frc);
        if (f->nangle > 0) orc_angles_f32(n, pos4, box, boxi, al, alm, pitch, f->ang1, f->ang2, frc);
        if (p->enstype == 1) {
            float scale = orc_berendsen_scale(p->dt, 0.01f, p->temper_0, temper);
            orc_leapfrog_nvt_f32(n, pos4, vel4, frc, p->dt, scale, box, boxi, 256, part);
            float ks;
            if (exact_ke) { ks = 0.0f; for (int b = 0; b < nblk; b++) ks += part[b]; }
            else ks = orc_ke_sum_ref(nblk, part);
            temper = orc_temperature_ref(ks, n);
        } else {
            orc_leapfrog_nve_f32(n, pos4, vel4, frc, p->dt, box, boxi);
        }
        if (temps_out) temps_out[t] = temper;
    }
    if (temper_io) *temper_io = temper;
    if (force4_out) memcpy(force4_out, frc, sizeof(float) * 4 * (size_t)n);
    rc = builds;
done:
    if (rc < 0) *have_list = 0;
    if (own) { free(nnl); free(nnm); free(pold); }
    free(excl); free(frc); free(part);
    free(bl); free(blm); free(al); free(alm);
    return rc;
}

static void plain_forces(const orc_params *p, const orc_ffield *f, int n, const double *x,
                         const int *itype, const float *q, const float box[3], const unsigned *excl,
                         float *pos4tmp, double *f4, double *ep, double *fout, double *pe)
{
    for (int i = 0; i < n; i++) {
        pos4tmp[4 * i] = (float)x[3 * i];
        pos4tmp[4 * i + 1] = (float)x[3 * i + 1];
        pos4tmp[4 * i + 2] = (float)x[3 * i + 2];
        pos4tmp[4 * i + 3] = 0.0f;
    }
    /* The plain form evaluates forces at the FP64 positions: the float copy
     * above only serves the list-free kernel's interface, so use FP64 deltas. */
    int kind = p->lkspace == 0 ? 0 : 1;
    pairmodel m;
    pairmodel_init(&m, kind, 0, p->rcutsq, p->reacf, p->alfa);
    const double qfac = (double)ORC_QFAC;
    const double L[3] = {box[0], box[1], box[2]};
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; i++) {
        double fx = 0, fy = 0, fz = 0, u = 0;
        for (int j = 0; j < n; j++) {
            if (j == i || is_excluded(excl, i, j)) continue;
            double d[3];
            for (int k = 0; k < 3; k++) { d[k] = x[3 * i + k] - x[3 * j + k]; d[k] -= L[k] * rint(d[k] / L[k]); }
            double rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (rsq > m.rcsq) continue;
            int t = itype[i] * f->ntype + itype[j];
            double ff, uu;
            pair_eval_f64(&m, rsq, qfac * (double)q[i] * (double)q[j], f->lj1[t], f->lj2[t], &ff, &uu);
            fx += ff * d[0]; fy += ff * d[1]; fz += ff * d[2];
            u += 0.5 * uu;
        }
        f4[4 * i] = fx; f4[4 * i + 1] = fy; f4[4 * i + 2] = fz; f4[4 * i + 3] = 0;
        ep[i] = u;
    }
    /* bonded terms on FP64 positions */
    for (int it = 0; it < f->nbonds; it++) {
        int t = f->bonds[3 * it] - 1, i = f->bonds[3 * it + 1] - 1, j = f->bonds[3 * it + 2] - 1;
        double d[3];
        for (int k = 0; k < 3; k++) { d[k] = x[3 * i + k] - x[3 * j + k]; d[k] -= L[k] * rint(d[k] / L[k]); }
        double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        double fa = (double)f->bnd1[t] * ((double)f->bnd2[t] / r - 1.0);
        for (int k = 0; k < 3; k++) { f4[4 * i + k] += fa * d[k]; f4[4 * j + k] -= fa * d[k]; }
        ep[i] += 0.25 * f->bnd1[t] * (r - f->bnd2[t]) * (r - f->bnd2[t]);
        ep[j] += 0.25 * f->bnd1[t] * (r - f->bnd2[t]) * (r - f->bnd2[t]);
    }
    for (int it = 0; it < f->nangle; it++) {
        int t = f->angles[4 * it] - 1, i = f->angles[4 * it + 1] - 1, j = f->angles[4 * it + 2] - 1,
            k = f->angles[4 * it + 3] - 1;
        double a[3], b[3];
        for (int c = 0; c < 3; c++) {
            a[c] = x[3 * i + c] - x[3 * j + c]; a[c] -= L[c] * rint(a[c] / L[c]);
            b[c] = x[3 * k + c] - x[3 * j + c]; b[c] -= L[c] * rint(b[c] / L[c]);
        }
        double aa = a[0] * a[0] + a[1] * a[1] + a[2] * a[2], bb = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
        double ab = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
        double c = ab / sqrt(aa * bb);
        if (c <= -0.9999999) c = -0.9999999;
        if (c >= 0.9999999) c = 0.9999999;
        double th = acos(c);
        double ff = (double)f->ang1[t] * (th - (double)f->ang2[t]) / sqrt(1.0 - c * c) / sqrt(aa * bb);
        for (int d = 0; d < 3; d++) {
            double fi = ff * (b[d] - ab / aa * a[d]), fk = ff * (a[d] - ab / bb * b[d]);
            f4[4 * i + d] += fi; f4[4 * k + d] += fk; f4[4 * j + d] -= fi + fk;
        }
        double u = 0.5 * f->ang1[t] * (th - f->ang2[t]) * (th - f->ang2[t]);
        ep[i] += u / 3; ep[j] += u / 3; ep[k] += u / 3;
    }
    double s = 0.0;
    for (int i = 0; i < n; i++) {
        fout[3 * i] = f4[4 * i]; fout[3 * i + 1] = f4[4 * i + 1]; fout[3 * i + 2] = f4[4 * i + 2];
        s += ep[i];
    }
    *pe = s;
}

int orc_md_plain_run(const orc_params *p, const orc_ffield *f, int n, double *x, double *v,
                     const int *itype, const float *q, const double *m, const float box[3],
                     int nsteps, int integrator, double *state_io, double *rec_out)
{
    unsigned *excl = (unsigned *)malloc(sizeof(unsigned) * 4 * (size_t)n);
    float *p4 = (float *)malloc(sizeof(float) * 4 * (size_t)n);
    double *f4 = (double *)malloc(sizeof(double) * 4 * (size_t)n);
    double *ep = (double *)malloc(sizeof(double) * (size_t)n);
    double *fr = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    double pe = 0.0;
    double xi = state_io ? state_io[0] : 0.0, eta = state_io ? state_io[1] : 0.0;
    double temper = (state_io && state_io[2] > 0) ? state_io[2] : p->temper_0;
    double dt = p->dt;
    int ndf = 3 * n - 3;
    double t0 = p->temper_0, kt = ORC_RGAS * t0;
    double tau = p->tau_t > 0 ? p->tau_t : 100.0;
    double qnh = ndf * kt * tau * tau;
    orc_build_exclusions(n, f->nbonds, f->bonds, excl);
    plain_forces(p, f, n, x, itype, q, box, excl, p4, f4, ep, fr, &pe);
    for (int t = 0; t < nsteps; t++) {
        if (integrator == 0) {
            double scale = 1.0;
            if (p->enstype == 1) scale = sqrt(1.0 + dt / tau * (t0 / temper - 1.0));
            orc_leapfrog_f64(n, x, v, fr, m, dt, scale, box);
            plain_forces(p, f, n, x, itype, q, box, excl, p4, f4, ep, fr, &pe);
            temper = 2.0 * orc_kinetic_f64(n, v, m) / (ndf * ORC_RGAS);
        } else {
            if (integrator == 2) orc_nh_half_f64(n, v, m, dt, t0, qnh, ndf, &xi, &eta);
            orc_vv_kick_f64(n, v, fr, m, 0.5 * dt);
            orc_vv_drift_f64(n, x, v, dt, box);
            plain_forces(p, f, n, x, itype, q, box, excl, p4, f4, ep, fr, &pe);
            orc_vv_kick_f64(n, v, fr, m, 0.5 * dt);
            if (integrator == 2) orc_nh_half_f64(n, v, m, dt, t0, qnh, ndf, &xi, &eta);
        }
        if (rec_out) {
            double ke = orc_kinetic_f64(n, v, m);
            double cons = ke + pe;
            if (integrator == 2) cons += 0.5 * qnh * xi * xi + ndf * kt * eta;
            rec_out[3 * t] = ke; rec_out[3 * t + 1] = pe; rec_out[3 * t + 2] = cons;
        }
    }
    if (state_io) { state_io[0] = xi; state_io[1] = eta; state_io[2] = temper; state_io[3] = pe; }
    free(excl); free(p4); free(f4); free(ep); free(fr);
    return 0;
}


/* Pair and bond forces of the plain form (FP64, all pairs, double box) with
 * the virial W = sum over atoms of ff r^2 (every pair counted from both
 * atoms, as the reference's force.w); angles are not supported here. */
static double npt_forces(const orc_params *p, const orc_ffield *f, int n, const double *x, const int *itype,
                         const float *q, const double L[3], const unsigned *excl, double *fr)
{
    int kind = p->lkspace == 0 ? 0 : 1;
    pairmodel m;
    pairmodel_init(&m, kind, 0, p->rcutsq, p->reacf, p->alfa);
    const double qfac = (double)ORC_QFAC;
    double W = 0.0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : W)
    for (int i = 0; i < n; i++) {
        double fx = 0, fy = 0, fz = 0;
        for (int j = 0; j < n; j++) {
            if (j == i || is_excluded(excl, i, j)) continue;
            double d[3];
            for (int k = 0; k < 3; k++) { d[k] = x[3 * i + k] - x[3 * j + k]; d[k] -= L[k] * rint(d[k] / L[k]); }
            double rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (rsq > m.rcsq) continue;
            int t = itype[i] * f->ntype + itype[j];
            double ff, uu;
            pair_eval_f64(&m, rsq, qfac * (double)q[i] * (double)q[j], f->lj1[t], f->lj2[t], &ff, &uu);
            fx += ff * d[0]; fy += ff * d[1]; fz += ff * d[2];
            W += ff * rsq;
        }
        fr[3 * i] = fx; fr[3 * i + 1] = fy; fr[3 * i + 2] = fz;
    }
    for (int it = 0; it < f->nbonds; it++) {
        int t = f->bonds[3 * it] - 1, i = f->bonds[3 * it + 1] - 1, j = f->bonds[3 * it + 2] - 1;
        double d[3];
        for (int k = 0; k < 3; k++) { d[k] = x[3 * i + k] - x[3 * j + k]; d[k] -= L[k] * rint(d[k] / L[k]); }
        double rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        double fa = (double)f->bnd1[t] * ((double)f->bnd2[t] / sqrt(rsq) - 1.0);
        for (int k = 0; k < 3; k++) { fr[3 * i + k] += fa * d[k]; fr[3 * j + k] -= fa * d[k]; }
        W += 2.0 * fa * rsq;
    }
    return W;
}

int orc_md_plain_npt(const orc_params *p, const orc_ffield *f, int n, double *x, double *v, const int *itype,
                     const float *q, const double *m, double box[3], int nsteps, double p0, double mu_k,
                     double mu_max, double *rec_out)
{
    if (f->nangle > 0) return -1;
    unsigned *excl = (unsigned *)malloc(sizeof(unsigned) * 4 * (size_t)n);
    double *fr = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    orc_build_exclusions(n, f->nbonds, f->bonds, excl);
    const double dt = p->dt, t0 = p->temper_0, tau = p->tau_t > 0 ? p->tau_t : 100.0;
    const int ndf = 3 * n - 3;
    double L[3] = {box[0], box[1], box[2]};
    double W = npt_forces(p, f, n, x, itype, q, L, excl, fr);
    double temper = t0, mu_next = 1.0;
    for (int t = 0; t < nsteps; t++) {
        const double scale = sqrt(1.0 + dt / tau * (t0 / temper - 1.0));
        double Ln[3];
        for (int k = 0; k < 3; k++) Ln[k] = L[k] * mu_next;
        double ke = 0.0;
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) {
                double vv = (v[3 * i + k] + fr[3 * i + k] * dt / m[i]) * scale;
                v[3 * i + k] = vv;
                double xx = (x[3 * i + k] + vv * dt) * mu_next;
                xx -= Ln[k] * trunc(xx * 2.0 / Ln[k]);
                x[3 * i + k] = xx;
                ke += 0.5 * m[i] * vv * vv;
            }
        temper = 2.0 * ke / (ndf * ORC_RGAS);
        const double P = (2.0 * ke + 0.5 * W) / (3.0 * L[0] * L[1] * L[2]);
        const double mu_used = mu_next;
        mu_next = 1.0 - mu_k * (p0 - P);
        mu_next = fmin(fmax(mu_next, 1.0 - mu_max), 1.0 + mu_max);
        for (int k = 0; k < 3; k++) L[k] = Ln[k];
        W = npt_forces(p, f, n, x, itype, q, L, excl, fr);
        if (rec_out) {
            rec_out[4 * t] = L[0]; rec_out[4 * t + 1] = P; rec_out[4 * t + 2] = temper; rec_out[4 * t + 3] = mu_used;
        }
    }
    for (int k = 0; k < 3; k++) box[k] = L[k];
    free(excl); free(fr);
    return 0;
}

/* ====================================================================== */
/* Adjoint of velocity-Verlet NVE (FP64, all pairs).                      */
/*                                                                        */
/* Forward, per step: v_h = v + c F(x); x' = x + dt v_h; v' = v_h + c F(x'),  */
/* c = dt/(2 m).  With P = dL/dx and u_m = dL/dv_h(m), reverse mode gives */
/*   u_m  = u_{m+1} + dt P_{m+1}            (u_K = 0)                      */
/*   P_m  = P_{m+1} + dO_m/dx_m + f_m c J(x_m) u_m                          */
/*   dL/dtheta += f_m c (dF(x_m)/dtheta) . u_m                             */
/* with f_m = 2 for 1 <= m <= K-1 (F(x_m) enters two half kicks, both with */
/* the same adjoint vector u_m) and f_0 = 1; J = dF/dx is symmetric:       */
/* (J w)_i = sum_j [ff (w_i - w_j) + g (d.(w_i - w_j)) d], g = (dff/dr)/r. */
/* ====================================================================== */

typedef struct {
    double rc, rcsq, alpha, spi, W, ec_c, p, rc6i, rc12i;
} adjmodel;

static void adjmodel_init(adjmodel *m, double rcutsq, double alfa)
{
    m->rcsq = rcutsq;
    m->rc = sqrt(rcutsq);
    m->alpha = alfa;
    m->p = (double)ORC_PEX * alfa;
    m->spi = 2.0 / sqrt(3.14159265358979323846) * alfa;
    double ec = erfc_as(alfa * m->rc);
    m->W = ec / m->rc + m->spi * exp(-alfa * alfa * rcutsq);
    m->ec_c = ec / m->rc;
    double rc2i = 1.0 / rcutsq;
    m->rc6i = rc2i * rc2i * rc2i;
    m->rc12i = m->rc6i * m->rc6i;
}

typedef struct {
    double ff, g, ffc, uc, ulj1, ulj2, flj1, flj2;
} adjterm;

/* Force factor ff (F_i = ff d), g = (dff/dr)/r, the Coulomb parts for the
 * charge-scale derivative, and the derivatives of u and ff with respect to
 * lj1 and lj2; qq includes qfac. */
static inline void adj_pair(const adjmodel *m, double rsq, double qq, double l1, double l2,
                            adjterm *o)
{
    double r = sqrt(rsq), ri = 1.0 / r, ri2 = ri * ri;
    double a = m->alpha;
    double t = 1.0 / (1.0 + m->p * r);
    double P = ((((double)ORC_A5 * t + (double)ORC_A4) * t + (double)ORC_A3) * t + (double)ORC_A2) * t + (double)ORC_A1;
    double dPt = (((5.0 * (double)ORC_A5 * t + 4.0 * (double)ORC_A4) * t + 3.0 * (double)ORC_A3) * t +
                  2.0 * (double)ORC_A2) * t + (double)ORC_A1;   /* d(tP)/dt */
    double e = exp(-a * a * rsq);
    double E = P * t * e;                                     /* A&S erfc(a r) */
    double dE = dPt * (-m->p * t * t) * e + P * t * (-2.0 * a * a * r) * e;
    double h = m->spi * e + E * ri;
    double dh = m->spi * (-2.0 * a * a * r) * e + dE * ri - E * ri2;
    double fc = qq * (h - m->W) * ri2;
    double dfc = qq * (dh * ri2 - 2.0 * (h - m->W) * ri2 * ri);
    double ri6 = ri2 * ri2 * ri2, ri8 = ri6 * ri2, ri14 = ri6 * ri8;
    double flj = l1 * ri14 - l2 * ri8;
    double dflj = -14.0 * l1 * ri14 * ri + 8.0 * l2 * ri8 * ri;
    o->ff = fc + flj;
    o->g = (dfc + dflj) * ri;
    o->ffc = fc;
    o->uc = qq * (E * ri - m->ec_c + m->W * log(r / m->rc));
    o->ulj1 = (ri6 * ri6 - m->rc12i) / 12.0;
    o->ulj2 = -(ri6 - m->rc6i) / 6.0;
    o->flj1 = ri14;
    o->flj2 = -ri8;
}

static inline void adj_delta(const double *x, int i, int j, const double *L, double d[3])
{
    for (int k = 0; k < 3; k++) {
        d[k] = x[3 * i + k] - x[3 * j + k];
        d[k] -= L[k] * rint(d[k] / L[k]);
    }
}

/* Whether atoms i and j are bonded (excluded from the pair terms). */
static int adj_excluded(const orc_adj_cfg *c, int i, int j)
{
    for (int b = 0; b < c->nbonds; b++) {
        const int *e = c->bonds + 3 * b;
        if ((e[1] == i && e[2] == j) || (e[1] == j && e[2] == i)) return 1;
    }
    return 0;
}

/* Bonded forces added to F and their energy (bonded_forces.cu:34-193 in
 * FP64: the same force expressions, cos(theta) clamped to +-0.9999999). */
static double adj_bonded(const orc_adj_cfg *c, const double *x, double *F)
{
    double U = 0.0;
    for (int b = 0; b < c->nbonds; b++) {
        const int *e = c->bonds + 3 * b;
        const int i = e[1], j = e[2];
        double d[3];
        adj_delta(x, i, j, c->box, d);
        const double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        const double kk = c->bnd1[e[0]], r0 = c->bnd2[e[0]];
        const double fa = kk * (r0 / r - 1.0);
        for (int k = 0; k < 3; k++) {
            F[3 * i + k] += fa * d[k];
            F[3 * j + k] -= fa * d[k];
        }
        U += 0.5 * kk * (r - r0) * (r - r0);
    }
    for (int a = 0; a < c->nangles; a++) {
        const int *e = c->angles + 4 * a;
        const int i = e[1], j = e[2], k2 = e[3];
        double av[3], bv[3];
        adj_delta(x, i, j, c->box, av);
        adj_delta(x, k2, j, c->box, bv);
        const double ai = 1.0 / sqrt(av[0] * av[0] + av[1] * av[1] + av[2] * av[2]);
        const double bi = 1.0 / sqrt(bv[0] * bv[0] + bv[1] * bv[1] + bv[2] * bv[2]);
        const double ab = av[0] * bv[0] + av[1] * bv[1] + av[2] * bv[2];
        double cang = ab * ai * bi;
        cang = cang < -0.9999999 ? -0.9999999 : (cang > 0.9999999 ? 0.9999999 : cang);
        const double th = acos(cang), k1 = c->ang1[e[0]], th0 = c->ang2[e[0]];
        const double ff = k1 * (th - th0) / sqrt(1.0 - cang * cang) * ai * bi;
        const double aa = ab * ai * ai, bb = ab * bi * bi;
        for (int q = 0; q < 3; q++) {
            const double gi = bv[q] - aa * av[q];   /* end atom i */
            const double gk = av[q] - bb * bv[q];   /* end atom k */
            F[3 * i + q] += ff * gi;
            F[3 * k2 + q] += ff * gk;
            F[3 * j + q] -= ff * (gi + gk);         /* the centre */
        }
        U += 0.5 * k1 * (th - th0) * (th - th0);
    }
    return U;
}

/* Forces and potential energy at x (all pairs inside rc). */
static double adj_forces(const orc_adj_cfg *c, const adjmodel *m, const int *itype, const double *q,
                         const double *lj1, const double *lj2, const double *x, double *F)
{
    const int n = c->natom, nt = c->ntype;
    const double qfac = (double)ORC_QFAC;
    double *ui = (double *)calloc((size_t)n + 1, sizeof(double));
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; i++) {
        double f0 = 0, f1 = 0, f2 = 0, U = 0.0;
        for (int j = 0; j < n; j++) {
            if (j == i || (c->nbonds && adj_excluded(c, i, j))) continue;
            double d[3];
            adj_delta(x, i, j, c->box, d);
            double rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (rsq > m->rcsq) continue;
            int t = itype[i] * nt + itype[j];
            adjterm o;
            adj_pair(m, rsq, qfac * q[i] * q[j], lj1[t], lj2[t], &o);
            f0 += o.ff * d[0]; f1 += o.ff * d[1]; f2 += o.ff * d[2];
            U += 0.5 * (o.uc + lj1[t] * o.ulj1 + lj2[t] * o.ulj2);
        }
        F[3 * i] = f0; F[3 * i + 1] = f1; F[3 * i + 2] = f2;
        ui[i] = U;
    }
    double U = 0.0;   /* fixed order: the result does not depend on the thread count */
    for (int i = 0; i < n; i++) U += ui[i];
    free(ui);
    return U + adj_bonded(c, x, F);
}

static double adj_rdf_norm(const orc_adj_cfg *c, const int *itype, int b)
{
    int na = 0, nb = 0;
    for (int i = 0; i < c->natom; i++) {
        na += itype[i] == c->rdf_a;
        nb += itype[i] == c->rdf_b;
    }
    double V = c->box[0] * c->box[1] * c->box[2];
    double rb = (b + 0.5) * c->rdf_dr;
    return V / ((double)na * (double)nb * 4.0 * 3.14159265358979323846 * rb * rb);
}

/* Adds the smoothed RDF of frame x to g (nbins). */
static void adj_rdf_add(const orc_adj_cfg *c, const int *itype, const double *x, const double *norm,
                        double *g)
{
    const int n = c->natom, nb = c->nbins;
    const double s = c->rdf_sigma, rmax = nb * c->rdf_dr + 5.0 * s;
    const double kn = 1.0 / (sqrt(2.0 * 3.14159265358979323846) * s);
    for (int i = 0; i < n; i++) {
        if (itype[i] != c->rdf_a) continue;
        for (int j = 0; j < n; j++) {
            if (j == i || itype[j] != c->rdf_b || (c->nbonds && adj_excluded(c, i, j))) continue;
            double d[3];
            adj_delta(x, i, j, c->box, d);
            double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            if (r >= rmax) continue;
            for (int b = 0; b < nb; b++) {
                double y = (b + 0.5) * c->rdf_dr - r;
                if (fabs(y) > 5.0 * s) continue;
                g[b] += norm[b] * kn * exp(-0.5 * y * y / (s * s));
            }
        }
    }
}

/* Gradient of sum_b e_b g_b(x) with respect to x, added to G. */
static void adj_rdf_grad(const orc_adj_cfg *c, const int *itype, const double *x, const double *norm,
                         const double *e, double *G)
{
    const int n = c->natom, nb = c->nbins;
    const double s = c->rdf_sigma, rmax = nb * c->rdf_dr + 5.0 * s;
    const double kn = 1.0 / (sqrt(2.0 * 3.14159265358979323846) * s);
    for (int i = 0; i < n; i++) {
        if (itype[i] != c->rdf_a) continue;
        for (int j = 0; j < n; j++) {
            if (j == i || itype[j] != c->rdf_b || (c->nbonds && adj_excluded(c, i, j))) continue;
            double d[3];
            adj_delta(x, i, j, c->box, d);
            double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            if (r >= rmax) continue;
            double coef = 0.0;   /* sum_b e_b dg_b/dr */
            for (int b = 0; b < nb; b++) {
                double y = (b + 0.5) * c->rdf_dr - r;
                if (fabs(y) > 5.0 * s) continue;
                coef += e[b] * norm[b] * kn * exp(-0.5 * y * y / (s * s)) * y / (s * s);
            }
            for (int k = 0; k < 3; k++) {
                G[3 * i + k] += coef * d[k] / r;
                G[3 * j + k] -= coef * d[k] / r;
            }
        }
    }
}

/* The forward trajectory: frames (K+1) x 3N, mean PE, gbar. */
static void adj_forward(const orc_adj_cfg *c, const adjmodel *m, const int *itype, const double *q,
                        const double *mass, const double *lj1, const double *lj2, const double *x0,
                        const double *v0, double *frames, double *pe_mean, double *gbar,
                        const double *norm)
{
    const int n = c->natom, K = c->nsteps;
    double *x = (double *)malloc(sizeof(double) * 3 * n), *v = (double *)malloc(sizeof(double) * 3 * n);
    double *F = (double *)malloc(sizeof(double) * 3 * n);
    memcpy(x, x0, sizeof(double) * 3 * n);
    memcpy(v, v0, sizeof(double) * 3 * n);
    for (int b = 0; b < c->nbins; b++) gbar[b] = 0.0;
    double usum = adj_forces(c, m, itype, q, lj1, lj2, x, F);
    adj_rdf_add(c, itype, x, norm, gbar);
    if (frames) memcpy(frames, x, sizeof(double) * 3 * n);
    for (int s = 0; s < K; s++) {
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) {
                v[3 * i + k] += 0.5 * c->dt / mass[i] * F[3 * i + k];
                x[3 * i + k] += c->dt * v[3 * i + k];
                x[3 * i + k] -= c->box[k] * trunc(2.0 * x[3 * i + k] / c->box[k]);
            }
        usum += adj_forces(c, m, itype, q, lj1, lj2, x, F);
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) v[3 * i + k] += 0.5 * c->dt / mass[i] * F[3 * i + k];
        adj_rdf_add(c, itype, x, norm, gbar);
        if (frames) memcpy(frames + (size_t)3 * n * (s + 1), x, sizeof(double) * 3 * n);
    }
    for (int b = 0; b < c->nbins; b++) gbar[b] /= (K + 1);
    *pe_mean = usum / (K + 1);
    free(x); free(v); free(F);
}

double orc_adj_loss(const orc_adj_cfg *c, const int *itype, const double *q, const double *mass,
                    const double *lj1, const double *lj2, const double *x0, const double *v0,
                    const double *target, double *gbar_out, double *pe_mean_out)
{
    adjmodel m;
    adjmodel_init(&m, c->rcutsq, c->alfa);
    double *norm = (double *)calloc((size_t)c->nbins + 1, sizeof(double));
    double *gbar = (double *)malloc(sizeof(double) * c->nbins);
    for (int b = 0; b < c->nbins; b++) norm[b] = adj_rdf_norm(c, itype, b);
    double pe = 0.0;
    adj_forward(c, &m, itype, q, mass, lj1, lj2, x0, v0, NULL, &pe, gbar, norm);
    double L = c->w_pe * pe / c->natom;
    for (int b = 0; b < c->nbins; b++) {
        double t = target ? target[b] : 0.0;
        L += c->w_rdf * (gbar[b] - t) * (gbar[b] - t);
    }
    if (gbar_out) memcpy(gbar_out, gbar, sizeof(double) * c->nbins);
    if (pe_mean_out) *pe_mean_out = pe;
    free(norm); free(gbar);
    return L;
}

double orc_adj_grad(const orc_adj_cfg *c, const int *itype, const double *q, const double *mass,
                    const double *lj1, const double *lj2, const double *x0, const double *v0,
                    const double *target, double *dlj1, double *dlj2, double *dlns,
                    double *gbar_out)
{
    const int n = c->natom, K = c->nsteps, nt = c->ntype, nb = c->nbins;
    adjmodel m;
    adjmodel_init(&m, c->rcutsq, c->alfa);
    double *norm = (double *)calloc((size_t)nb + 1, sizeof(double));
    double *gbar = (double *)malloc(sizeof(double) * nb);
    double *e = (double *)malloc(sizeof(double) * nb);
    double *frames = (double *)malloc(sizeof(double) * 3 * n * (size_t)(K + 1));
    double *P = (double *)calloc(3 * (size_t)n, sizeof(double));
    double *U = (double *)calloc(3 * (size_t)n, sizeof(double));
    double *w = (double *)malloc(sizeof(double) * 3 * n);
    double *F = (double *)malloc(sizeof(double) * 3 * n);
    for (int b = 0; b < nb; b++) norm[b] = adj_rdf_norm(c, itype, b);
    double pe = 0.0;
    adj_forward(c, &m, itype, q, mass, lj1, lj2, x0, v0, frames, &pe, gbar, norm);
    double L = c->w_pe * pe / n;
    for (int b = 0; b < nb; b++) {
        double t = target ? target[b] : 0.0;
        L += c->w_rdf * (gbar[b] - t) * (gbar[b] - t);
        e[b] = c->w_rdf * 2.0 * (gbar[b] - t) / (K + 1);
    }
    for (int k = 0; k < nt * nt; k++) { dlj1[k] = 0.0; dlj2[k] = 0.0; }
    *dlns = 0.0;
    const double wpe = c->w_pe / ((double)(K + 1) * n);
    const double qfac = (double)ORC_QFAC;
    for (int mfr = K; mfr >= 0; mfr--) {
        const double *x = frames + (size_t)3 * n * mfr;
        if (mfr < K) {
            double fac = mfr >= 1 ? 2.0 : 1.0;
            for (int i = 0; i < 3 * n; i++) {
                U[i] += c->dt * P[i];
                w[i] = fac * 0.5 * c->dt / mass[i / 3] * U[i];
            }
        }
        /* observable gradient (PE: -F; RDF) and, below the last frame, J w
         * and the parameter terms; explicit dU/dtheta for every frame */
        adj_forces(c, &m, itype, q, lj1, lj2, x, F);
        for (int i = 0; i < 3 * n; i++) P[i] -= wpe * F[i];
        adj_rdf_grad(c, itype, x, norm, e, P);
        for (int i = 0; i < n; i++)
            for (int j = i + 1; j < n; j++) {
                if (c->nbonds && adj_excluded(c, i, j)) continue;
                double d[3];
                adj_delta(x, i, j, c->box, d);
                double rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                if (rsq > m.rcsq) continue;
                int tij = itype[i] * nt + itype[j], tji = itype[j] * nt + itype[i];
                adjterm o;
                adj_pair(&m, rsq, qfac * q[i] * q[j], lj1[tij], lj2[tij], &o);
                /* explicit derivative of the mean PE (each table entry carries half a pair) */
                dlj1[tij] += 0.5 * wpe * o.ulj1; dlj1[tji] += 0.5 * wpe * o.ulj1;
                dlj2[tij] += 0.5 * wpe * o.ulj2; dlj2[tji] += 0.5 * wpe * o.ulj2;
                *dlns += wpe * 2.0 * o.uc;
                if (mfr == K) continue;
                double dwi = d[0] * w[3 * i] + d[1] * w[3 * i + 1] + d[2] * w[3 * i + 2];
                double dwj = d[0] * w[3 * j] + d[1] * w[3 * j + 1] + d[2] * w[3 * j + 2];
                double dd = dwi - dwj;
                for (int k = 0; k < 3; k++) {
                    double jw = o.ff * (w[3 * i + k] - w[3 * j + k]) + o.g * dd * d[k];
                    P[3 * i + k] += jw;
                    P[3 * j + k] -= jw;
                }
                /* dynamics term: row i uses entry (ti,tj) with d.w_i, row j entry (tj,ti) with -d.w_j */
                dlj1[tij] += o.flj1 * dwi; dlj1[tji] -= o.flj1 * dwj;
                dlj2[tij] += o.flj2 * dwi; dlj2[tji] -= o.flj2 * dwj;
                *dlns += 2.0 * o.ffc * dd;
            }
        /* bonded J w by central differences of the bonded forces along w
         * (step 1e-6 A over the largest component of w) */
        if (mfr < K && (c->nbonds || c->nangles)) {
            double wmax = 0.0;
            for (int i = 0; i < 3 * n; i++) wmax = fmax(wmax, fabs(w[i]));
            if (wmax > 0.0) {
                const double h = 1e-6 / wmax;
                double *xp = (double *)malloc(sizeof(double) * 3 * n);
                double *fp = (double *)calloc(3 * (size_t)n, sizeof(double));
                double *fm = (double *)calloc(3 * (size_t)n, sizeof(double));
                for (int i = 0; i < 3 * n; i++) xp[i] = x[i] + h * w[i];
                adj_bonded(c, xp, fp);
                for (int i = 0; i < 3 * n; i++) xp[i] = x[i] - h * w[i];
                adj_bonded(c, xp, fm);
                for (int i = 0; i < 3 * n; i++) P[i] += (fp[i] - fm[i]) / (2.0 * h);
                free(xp); free(fp); free(fm);
            }
        }
    }
    if (gbar_out) memcpy(gbar_out, gbar, sizeof(double) * nb);
    free(norm); free(gbar); free(e); free(frames); free(P); free(U); free(w); free(F);
    return L;
}
