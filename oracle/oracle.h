/*
 * oracle.h -- CPU restatement of md_gpu's per-step force-and-integrate path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path in
 * md_gpu_gb300/: the parity tests, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py call it, nothing in the product does.
 *
 * Two arithmetic modes are provided for every hot-path function:
 *   *_f32  "as written": FP32 with the reference's operation order and no
 *          FMA contraction (build with -ffp-contract=off).  Device intrinsics
 *          are modelled as rsqrtf(x) = 1/sqrtf(x), __fdividef(a,b) = a/b,
 *          exp2f/acosf = libm.  Pinned bit-exactly against the reference's own
 *          kernel sources run on the CPU (oracle/ref_emu, tests/golden).
 *   *_f64  the "plain form": the same formulas in FP64 (positions, charges
 *          and parameter tables as given), used for error metrics.
 *
 * Layouts follow the reference: float4 records pos = (x,y,z,w) with
 * w = itype + 0.1(q+5) (config.cu:34), vel = (vx,vy,vz,m*1e4),
 * force = (fx,fy,fz,6*virial); neighbour lists column-major
 * nnlist[i + pitch*k] with pitch = ceil(N/256)*256 (gpu_properties.cu:54,
 * neighborlist.cu:284); bonded lists bndlist[i + pitch*k] = (j,type),
 * anglist[i + pitch*k] = (role,other1,other2,type) (forces.cu:113-179).
 */
#ifndef MD_ORACLE_H
#define MD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAXTYPE 8

/* Run parameters from <name>.inp (simulation.cu:58-105). */
typedef struct {
    int enstype;            /* 0 nve, 1 nvt, 2 npt */
    float temper_0, press_0;
    int timeq, timrun, timprn;
    float dt;
    float rcutsq;           /* squared cutoff, as simulation.cu:96 */
    int lkspace;            /* 0 reaction field, 1 Wolf, 2 Ewald (alpha only) */
    float reacf;            /* 2(eps-1)/(2eps+1)/rc^3, simulation.cu:86 */
    float alfa;
    int kmax;
    float skin;
    int nmaxlist;
    float rdel;
    /* extension lines (absent from reference files; defaults otherwise) */
    float tau_t;            /* thermostat time constant, fs (default 100) */
    int integrator;         /* 0 leapfrog (reference default), 1 VV, 2 NH-VV */
} orc_params;

/* Force field from <name>.fld (simulation.cu:144-264). */
typedef struct {
    int ntype;
    int nt[ORC_MAXTYPE];
    char name[ORC_MAXTYPE][16];
    float mass[ORC_MAXTYPE];       /* g/mol * 1e4, simulation.cu:177 */
    float charge[ORC_MAXTYPE];
    float lj1[ORC_MAXTYPE * ORC_MAXTYPE];  /* [i*ntype + j], 48 eps sig^12 or 12A */
    float lj2[ORC_MAXTYPE * ORC_MAXTYPE];  /* 24 eps sig^6 or 6B */
    int tbonds;
    float bnd1[ORC_MAXTYPE], bnd2[ORC_MAXTYPE];   /* 2k, r0 */
    int tangle;
    float ang1[ORC_MAXTYPE], ang2[ORC_MAXTYPE];   /* 2k, theta0 [rad] */
    int nbonds, nangle;
    int *bonds;    /* nbonds x 3: type, i, j  (1-based, as in the file) */
    int *angles;   /* nangle x 4: type, i, j(centre), k (1-based) */
} orc_ffield;

/* Configuration from <name>.cfg (simulation.cu:278-316). */
typedef struct {
    int natom, cftyp;
    float box[3], boxi[3];
    int *itype;     /* 0-based */
    float *q;       /* charge as read */
    float *pos;     /* 3N */
    float *vel;     /* 3N */
    float *mass;    /* N, g/mol * 1e4 */
} orc_config;

/* ---- input files ---- */
int orc_read_inp(const char *path, orc_params *p);
int orc_read_fld(const char *path, orc_ffield *f);
int orc_read_cfg(const char *path, const orc_ffield *f, orc_config *c);
void orc_free_fld(orc_ffield *f);
void orc_free_cfg(orc_config *c);
int orc_write_cfg(const char *path, const orc_config *c, const float *pos3, const float *vel3);

/* ---- packing and constants ---- */
void orc_pack_pos4(int n, const float *pos3, const int *itype, const float *q, float *pos4);
void orc_pack_vel4(int n, const float *vel3, const float *mass, float *vel4);
float orc_decode_q(float w);
int orc_pitch(int n);
float orc_rskinsq(float skin, float rcutsq);
float orc_rmaxdif(float skin);
void orc_wolf_consts(float alfa, float rcutsq, float out4[4]);

/* ---- neighbour list (neighborlist.cu) ---- */
int orc_build_exclusions(int n, int nbonds, const int *bonds, unsigned *excl4);
int orc_nlist_nsquared(int n, const float *pos4, const float box[3], const float boxi[3],
                       float rskinsq, const unsigned *excl4, int pitch, int nmax,
                       unsigned *nnlist, unsigned *nnlist_max);
int orc_nlist_check(int n, const float *pos4, const float *pos_old4, const float box[3],
                    const float boxi[3], float rmaxdif);

/* ---- cell assignment and space-filling-curve order ---- */
void orc_cell_dims(const float box[3], float rl, int ncell[3], float binlen[3]);
void orc_cell_index(int n, const float *pos4, const float box[3], const int ncell[3],
                    const float binlen[3], int *cell3);
unsigned long long orc_hilbert3(unsigned x, unsigned y, unsigned z, int bits);

/* ---- pair forces (pair_forces.cu) ---- */
void orc_pair_f32(int kind, int n, const float *pos4, const float box[3], const float boxi[3],
                  const unsigned *nnlist, const unsigned *nnlist_max, int pitch, int ntype,
                  const float *lj1, const float *lj2, float rcutsq, float reacf,
                  const float wc[4], float *force4);
void orc_pair_f64(int kind, int erfc_exact, int n, const float *pos4, const int *itype,
                  const float *q, const float box[3], const unsigned *nnlist,
                  const unsigned *nnlist_max, int pitch, int ntype, const float *lj1,
                  const float *lj2, float rcutsq, float reacf, float alfa,
                  double *force4, double *epot);
void orc_pair_allpairs_f64(int kind, int erfc_exact, int n, const float *pos4, const int *itype,
                           const float *q, const float box[3], int ntype, const float *lj1,
                           const float *lj2, float rcutsq, float reacf, float alfa,
                           const unsigned *excl4, double *force4, double *epot);
long long orc_count_pairs(int n, const float *pos4, const float box[3], float rcutsq,
                          const unsigned *excl4);

/* ---- bonded forces (bonded_forces.cu) ---- */
int orc_bond_lists(int n, int nbonds, const int *bonds, int pitch, unsigned *bndlist2,
                   unsigned *bndlist_max);
int orc_angle_lists(int n, int nangle, const int *angles, int pitch, unsigned *anglist4,
                    unsigned *anglist_max);
void orc_bonds_f32(int n, const float *pos4, const float box[3], const float boxi[3],
                   const unsigned *bndlist2, const unsigned *bndlist_max, int pitch,
                   const float *bnd1, const float *bnd2, float *force4);
void orc_angles_f32(int n, const float *pos4, const float box[3], const float boxi[3],
                    const unsigned *anglist4, const unsigned *anglist_max, int pitch,
                    const float *ang1, const float *ang2, float *force4);
void orc_bonds_f64(int n, const float *pos4, const float box[3], int nbonds, const int *bonds,
                   const float *bnd1, const float *bnd2, double *force4, double *epot);
void orc_angles_f64(int n, const float *pos4, const float box[3], int nangle, const int *angles,
                    const float *ang1, const float *ang2, double *force4, double *epot);

/* ---- integrators, as written (nve_leapfrog.cu, nvt_leapfrog_ber.cu, nve_vverlet.cu) ---- */
void orc_leapfrog_nve_f32(int n, float *pos4, float *vel4, const float *force4, float dt,
                          const float box[3], const float boxi[3]);
void orc_leapfrog_nvt_f32(int n, float *pos4, float *vel4, const float *force4, float dt,
                          float scale, const float box[3], const float boxi[3], int block,
                          float *ke_partials);
float orc_ke_sum_ref(int nblocks, const float *partials);
float orc_berendsen_scale(float dt, float tco, float temper_0, float temper);
float orc_temperature_ref(float ke_sum0, int n);
void orc_vv_pre_f32(int n, float *pos4, float *vel4, const float *force4, float dt,
                    const float box[3], const float boxi[3]);
void orc_vv_cor_f32(int n, float *vel4, const float *force4, float dt);

/* ---- integrators, plain FP64 (state arrays: x,v,f 3N; m N in g/mol*1e4) ---- */
void orc_wrap_f64(int n, double *x, const float box[3]);
double orc_kinetic_f64(int n, const double *v, const double *m);
void orc_leapfrog_f64(int n, double *x, double *v, const double *f, const double *m,
                      double dt, double scale, const float box[3]);
void orc_vv_kick_f64(int n, double *v, const double *f, const double *m, double half_dt);
void orc_vv_drift_f64(int n, double *x, const double *v, double dt, const float box[3]);
void orc_nh_half_f64(int n, double *v, const double *m, double dt, double t0, double q_nh,
                     int ndf, double *xi, double *eta);

/* ---- whole runs ---- */
/* The reference's step loop (runGPU.cu:69-104) in FP32 as written, with the
 * O(N^2) list rebuilt on the reference's displacement criterion.  Leapfrog
 * NVE (enstype 0) or Berendsen NVT (enstype 1; exact_ke != 0 replaces the
 * reference's single-block KE tree by a straight sum).  pos4/vel4 in/out.
 * Returns the number of list builds, or -1 on list overflow. */
int orc_md_ref_run(const orc_params *p, const orc_ffield *f, int n, float *pos4, float *vel4,
                   const float box[3], const float boxi[3], int nsteps, int exact_ke,
                   float *force4_out, float *temper_io, float *temps_out);
/* The same loop continuing a run across calls: the caller owns the list
 * (nnl: orc_pitch(n) * nmaxlist, nnm: orc_pitch(n), pold: 4n floats); with
 * *have_list == 0 the call first builds it (neighborlist_init,
 * neighborlist.cu:30-106) and sets *have_list, otherwise it continues with
 * the list of the previous call and rebuilds only on the displacement
 * criterion (neighborlist.cu:109-146), as the reference's loop does between
 * its steps.  Returns the builds made in this call, or -1 on overflow. */
int orc_md_ref_run_cont(const orc_params *p, const orc_ffield *f, int n, float *pos4, float *vel4,
                        const float box[3], const float boxi[3], int nsteps, int exact_ke,
                        unsigned *nnl, unsigned *nnm, float *pold, int *have_list,
                        float *force4_out, float *temper_io, float *temps_out);

/* FP64 plain-form NPT run: leapfrog with the Berendsen thermostat (the
 * previous step's temperature, tau_t) and the Berendsen barostat the library
 * runs (no reference implementation: npt_leapfrog_ber.cu never scales the
 * box).  Each step: v = (v + F dt/m) lambda; x = (x + v dt) mu_next, wrapped
 * into the box scaled by mu_next; P = (2 KE + W/2) / (3 V) with W = sum over
 * atoms of ff r^2 of the step's forces and V the box they saw; mu_next = 1 -
 * mu_k (p0 - P) clamped to 1 +- mu_max.  All pairs, FP64 positions and box,
 * pair and bond terms (returns -1 with angles).  box in/out (A); p0 in
 * kJ/mol/A^3; rec_out (may be NULL): per step Lx, P (kJ/mol/A^3), T, the mu
 * the step applied. */
int orc_md_plain_npt(const orc_params *p, const orc_ffield *f, int n, double *x, double *v, const int *itype,
                     const float *q, const double *m, double box[3], int nsteps, double p0, double mu_k,
                     double mu_max, double *rec_out);

/* FP64 plain-form run: integrator 0 leapfrog(+Berendsen if enstype 1),
 * 1 velocity Verlet NVE, 2 Nose-Hoover VV.  All-pairs forces inside rc
 * (cell-free O(N^2), for small N only).  Writes per-step total energy
 * records [ke, pe, conserved] to rec_out (3*nsteps) when non-NULL. */
int orc_md_plain_run(const orc_params *p, const orc_ffield *f, int n, double *x, double *v,
                     const int *itype, const float *q, const double *m, const float box[3],
                     int nsteps, int integrator, double *state_io, double *rec_out);

/* ---- adjoint of velocity-Verlet NVE (no reference counterpart) ----
 * One system, FP64, all pairs inside rc (O(N^2) per frame, small N only),
 * LJ + Wolf Coulomb with A&S 7.1.26 erfc, harmonic bonds and angles.  Frames m = 0..K are the initial
 * configuration and the K steps.  Loss
 *   L = w_pe <U>/N + w_rdf sum_b (gbar_b - t_b)^2,
 * <U> the frame average of the consistent potential energy, gbar the frame
 * average of the Gaussian-smoothed RDF of type pair (rdf_a, rdf_b):
 *   g_b = V/(N_a N_b 4 pi r_b^2) sum_{i in a, j in b} K(r_b - r_ij),
 *   r_b = (b + 1/2) dr, K a normalised Gaussian of width sigma.
 * Gradients are with respect to every LJ table entry lj1[a*nt+b], lj2[...]
 * (as used by the row of an atom of type a) and to the log of a common
 * charge scale (charges q -> s q at s = 1). */
typedef struct {
    int natom, ntype, nsteps;
    double box[3];
    double rcutsq, alfa, dt;
    double w_pe, w_rdf;
    int rdf_a, rdf_b, nbins;
    double rdf_dr, rdf_sigma;
    /* harmonic bonds and angles (0-based atoms; may be 0 / NULL): the bonded
     * pairs are excluded from the pair terms and from the RDF, as the
     * neighbour list excludes them; bnd1 = 2k, ang1 = 2k per type
     * (U = k (r - r0)^2, U = k (theta - theta0)^2, theta0 in rad) */
    int nbonds, nangles;
    const int *bonds;    /* type, i, j */
    const int *angles;   /* type, i, j (centre), k */
    const double *bnd1, *bnd2, *ang1, *ang2;
} orc_adj_cfg;

/* Forward run only: the loss; gbar (nbins) and the mean PE when non-NULL.
 * target may be NULL (zero). */
double orc_adj_loss(const orc_adj_cfg *c, const int *itype, const double *q, const double *mass,
                    const double *lj1, const double *lj2, const double *x0, const double *v0,
                    const double *target, double *gbar, double *pe_mean);
/* Forward run and the discrete adjoint: returns the loss and writes dlj1,
 * dlj2 (ntype*ntype) and dlns (1). */
double orc_adj_grad(const orc_adj_cfg *c, const int *itype, const double *q, const double *mass,
                    const double *lj1, const double *lj2, const double *x0, const double *v0,
                    const double *target, double *dlj1, double *dlj2, double *dlns,
                    double *gbar);

int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
