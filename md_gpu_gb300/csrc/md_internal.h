/*
 * md_internal.h -- device data layout and kernel launchers of libmdgpu_gb300.
 *
 * One md_ctx holds one system resident in HBM.  Atoms live in cell order:
 * every neighbour-list build bins the atoms into cells of side >= rl/2,
 * orders the cells along a 3-D Hilbert curve and permutes every per-atom
 * array into that order (ties inside a cell broken by original index, so the
 * order is deterministic).  perm[] maps sorted -> original index, iperm[] the
 * reverse; everything the caller sees is in original order.
 *
 * Per sorted atom s:
 *   x,v      FP64 SoA (x[0..N) y[N..2N) z[2N..3N)), the integrated state
 *   pos4     float4 (x, y, z, q): FP32 copy the force kernels read
 *   fx,fy,fz int64 fixed point (FX_SCALE units of kJ/mol/A): every force
 *            term adds into these, so the sum is order independent
 *   vir      float, sum of ff r^2 (the reference's force.w, 6 x virial)
 *   nl       neighbour list, one row of `cap` entries per atom
 *            (nl[s*cap + k]), entry = j | (type_j << 29); each row is padded
 *            to a multiple of 32 entries with the atom itself (r = 0, which
 *            the force kernel skips), so readers need no bounds predicate
 */
#ifndef MD_INTERNAL_H
#define MD_INTERNAL_H

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/md_gpu.h"

#define MD_MAXTYPE 8
#define MD_TYPE_SHIFT 29
#define MD_INDEX_MASK 0x1FFFFFFFu
#define MD_EXCL_NONE 0xFFFFFFFFu
#define MD_LIST_QUANTUM 32   /* list rows are padded to multiples of this */
#define FX_SCALE 4294967296.0      /* 2^32 */
#define FX_INV (1.0 / 4294967296.0)

/* Step control and thermodynamic state kept on the device (no host syncs
 * inside a step). */
struct md_devstate {
    int update;          /* neighbour-list rebuild requested this step */
    int list_overflow;   /* largest list length seen beyond capacity, or 0 */
    int builds;          /* neighbour-list builds so far */
    long long step;
    double temper;       /* temperature after the last step, K */
    double ke;           /* kinetic energy, kJ/mol */
    double pe;           /* potential energy (when computed), kJ/mol */
    double virial;       /* sum ff r^2 / 6 (when computed) */
    double xi, eta;      /* Nose-Hoover thermostat variable and its integral */
    double xi_a, eta_a;  /* the same after the first thermostat half step of a step */
    double vscale;       /* velocity scale pending from the last thermostat half step */
    double lambda;       /* last Berendsen scale */
    double lam_next;     /* Berendsen scale of the next leapfrog step */
    double kick_scale;   /* velocity scale applied by the next VV first half (NH: s2*s1) */
    unsigned blocks_done; /* blocks finished in the current reduction kernel */
    unsigned long long acc[3]; /* fixed-point KE (MD_KFIX), PE, sum ff r^2 (MD_EFIX) of the step */
    int cell_next;       /* next cell a list-building warp takes (reset after each build) */
    /* grid barrier of the one-kernel rebuild: arrivals and generation, each
     * on its own 128-byte line, so that the waiting blocks' polls of the
     * generation do not contend with the arrivals' atomics */
    alignas(128) unsigned bar_count;
    alignas(128) unsigned bar_gen;
    /* sticky device-side error code (1: a grid barrier timed out), read by
     * the one-kernel rebuild: on a line of its own, which nothing writes
     * unless a wait times out, so those reads never queue behind the
     * atomics on the lines above */
    alignas(128) int status;
};

/* Everything a kernel needs about the system, passed by value. */
struct md_kparams {
    int n, pitch, cap, ntype;
    float box[3], boxi[3];
    double boxd[3];
    double box2i[3];  /* 2/L, for the wrap x -= L trunc(2x/L) */
    float rcutsq, reacf, rskinsq, rmaxdif;
    float palfa, spiialfa, alfasq, wolf;
    int lkspace;
    int ncell[3];
    float binlen[3];
    int stencil[3];   /* cell range per axis: +-stencil, or -1 = all cells */
    int cell_shift;   /* 1: a stencil cell's periodic image fixes the min-image shift
                         (positions centered, stencil narrow enough) */
    float wlim[3];    /* 0.4999 L: |x| below it needs no periodic wrap */
    double dt;
    int centered;     /* 1: every position lies in [-L/2, L/2] on each axis */
};

/* One replica of a batch: its geometry, cutoffs, cell grid and thermostat
 * constants.  A batch keeps every replica's atoms in one contiguous range
 * (the same range in the original and in the sorted order, since a build
 * only reorders atoms inside their replica's cells) and its cells in one
 * contiguous range of ranks. */
struct md_rep {
    float box[3], boxi[3];
    double boxd[3], box2i[3];
    float wlim[3];
    float rcutsq, rskinsq, rmaxdif, reacf;
    float palfa, spiialfa, alfasq, wolf;
    float ucc, rc6i, rcinv;
    int ncell[3], stencil[3];
    float binlen[3];
    int cell_shift;
    int cell0, ncells;   /* first cell rank (= offset of its cell_rank table), cell count */
    int atom0, natom;
    int blk0, nblk;      /* its blocks of the MD_LA-atom integrator grid */
    int ablk0, anblk;    /* its blocks of the MD_ADJ_ATOMS-atom grid of the adjoint kernels */
    int ndf;
    double t0, q_nh, inv_ndfr, inv_q;   /* 1/(ndf R), 1/Q */
    /* Berendsen barostat (NPT): target pressure (kJ/mol/A^3), the factor
     * k of mu = 1 - k (p0 - P) (compressibility dt / (3 tau_p)), the
     * largest |mu - 1| of a step, and half the list radius the cell grid
     * must keep (binlen >= rl/2) */
    double p0, mu_k, mu_max;
    int npt;
    float rl_half;
};

/* Constants of the FP64 force law of one system or replica (the FP64 mode,
 * md_set_precision): cutoff, reaction-field or Wolf constants, the A&S erfc
 * coefficients widened from the reference's floats, box. */
struct md_p64 {
    int kind;   /* lkspace: 0 reaction field, 1 Wolf, 2 LJ + no Coulomb shift */
    double rcsq, rc, rcinv, rc6i, reacf, alpha, spi, pex, a[5], qfac, wolfw, ucc;
    double L[3], Li[3];
};
md_p64 md_make_p64(int lkspace, float rcutsq, float reacf, float alfa, const float box[3]);

/* Per-replica thermodynamic state of a batch (the fields md_devstate holds
 * for a single system). */
struct md_repstate {
    double temper, ke, pe, virial;
    double xi, eta, xi_a, eta_a;
    double vscale, lambda, lam_next, kick_scale;
    int builds;          /* neighbour-list builds of this replica */
    int pad;
    double mu_next;      /* NPT: box scale the next step applies */
    double mu_used;      /* NPT: box scale the last step applied */
    double pressure;     /* NPT: pressure of the last step, kJ/mol/A^3 */
};

/* Replica-aligned launch grids of a batch: for A atoms per block (A = 4 ..
 * 256, powers of two) block b covers atoms [tab[b].y, min(tab[b].y + A, end
 * of replica tab[b].x)). */
#define MD_NGRID 7
/* Integrator blocks: MD_LA atoms x 3 axes, one thread per (atom, axis). */
#define MD_LA 128
/* Atoms per block of the adjoint pair kernels. */
#define MD_ADJ_ATOMS 32
/* Fixed-point scales of the energy accumulators: kinetic energy 2^32 per
 * kJ/mol (|KE| < 2.1e9 kJ/mol per system), potential energy and virial 2^24
 * (|PE| < 5.4e11 kJ/mol). */
#define MD_KFIX 4294967296.0
#define MD_EFIX 16777216.0
inline int md_grid_index(int atoms_per_block)
{
    int k = 0;
    while ((4 << k) < atoms_per_block) k++;
    return k;
}

/* Smooth particle-mesh Ewald of a single system (k_pme.cu, md_set_pme). */
struct md_pme {
    int on = 0;
    int K[3] = {0, 0, 0};          /* grid points per axis (multiples of 8, >= 16) */
    int ncand[3] = {0, 0, 0};      /* cells per axis searched for one brick's atoms */
    float *grid = nullptr;         /* K0 K1 K2 reals: the charges, then the convolution */
    void *spec = nullptr;          /* K0 K1 (K2/2+1) complex: the half spectrum */
    float *infl = nullptr;         /* B(m) C(m) on the half spectrum */
    int4 *org = nullptr;           /* per sorted atom: spline origin (x, y, z) */
    float4 *wq = nullptr;          /* per sorted atom: offsets (x, y, z) and charge */
    int fwd = 0, inv = 0;          /* cuFFT plans (cufftHandle) */
    int plans = 0;                 /* plans created */
    int excl = 0;                  /* the system has excluded pairs to remove */
    int nsm = 1;
    float e_bg = 0.0f;             /* background energy of a net charge, per atom */
};

struct md_ctx {
    /* ---- host copy of the run ---- */
    int n = 0, ntype = 0, pitch = 0, cap = 0;
    float box[3] = {0, 0, 0}, boxi[3] = {0, 0, 0};
    int lkspace = 1, enstype = 0, integrator = 0, nmaxlist = 0, timprn = 1;
    float rcutsq = 0, reacf = 0, alfa = 0, skin = 0, temper_0 = 0, dt = 1, tau_t = 100, rdel = 0.02f;
    float wc[4] = {0, 0, 0, 0};
    float rskinsq = 0, rmaxdif = 0;
    float lj1[64], lj2[64];
    float bnd1[MD_MAXTYPE], bnd2[MD_MAXTYPE], ang1[MD_MAXTYPE], ang2[MD_MAXTYPE];
    float type_mass[MD_MAXTYPE];
    std::vector<int> itype;          /* original order, 0-based */
    std::vector<float> charge;
    std::vector<int> bonds;          /* type, i, j (0-based) */
    std::vector<int> angles;         /* type, i, j(centre), k (0-based) */
    std::vector<unsigned> excl_host; /* 4 per atom, the reference's slot rule */
    unsigned type_excl_mask[MD_MAXTYPE] = {0};
    int ncell[3] = {1, 1, 1}, ncells = 1;
    float binlen[3] = {0, 0, 0};
    int stencil[3] = {0, 0, 0};
    std::string last_error;

    /* ---- device ---- */
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;  /* captures the bodies of conditional graph nodes */
    bool own_stream = false;
    int device = 0;
    double *x = nullptr, *v = nullptr, *mass = nullptr;   /* sorted order */
    double *kick = nullptr;   /* dt/m * 2^-32: fixed-point force -> velocity change of one step */
    float4 *pos4 = nullptr, *pos_old = nullptr;
    float4 *pos4_alt = nullptr;     /* second position buffer of the fused step */
    int *type = nullptr, *perm = nullptr, *iperm = nullptr;
    long long *f = nullptr;                               /* 3*pitch, SoA */
    float *vir = nullptr, *epot = nullptr;
    unsigned *nl = nullptr;
    int *nl_n = nullptr;
    uint4 *excl_orig = nullptr, *excl_s = nullptr;
    int *cell_rank = nullptr, *cell_count = nullptr, *cell_start = nullptr, *cell_fill = nullptr;
    int *cell_lin = nullptr;                              /* rank -> linear cell index */
    int *cell_work = nullptr;                             /* cell ranks, most atoms first (list-build order) */
    int *key = nullptr, *src = nullptr;
    double *tmp_d = nullptr;                              /* 8*pitch scratch for permutation */
    float4 *tmp4 = nullptr;
    int *tmp_i = nullptr;                                 /* 3*pitch */
    /* bonded lists: original-space CSR (fixed) and sorted-space per-atom slots */
    int2 *bl_o = nullptr; int *bl_on = nullptr;           /* 4 per original atom */
    int4 *al_o = nullptr; int *al_on = nullptr;
    int2 *bl_s = nullptr; int *bl_sn = nullptr;           /* column-major, 4*pitch */
    int4 *al_s = nullptr; int *al_sn = nullptr;
    int has_bonds = 0, has_angles = 0;
    md_devstate *st = nullptr;
    md_thermo *rec = nullptr;                             /* device ring of records */
    double *rep_hist = nullptr;   /* batches: ring of per-replica (KE, PE, conserved) per step */
    int rec_cap = 0;              /* records in the ring (a power of two) */
    float *lj_dev = nullptr;                              /* lj1,lj2 interleaved (64 float2) */
    float *bonded_par = nullptr;                          /* bnd1,bnd2,ang1,ang2 (4x8) */
    unsigned *type_mask_dev = nullptr;

    /* graph of gsteps steps (energy on its first step when genergy) */
    cudaGraphExec_t gexec = nullptr;
    int gsteps = 0;
    int genergy = 0;
    const float4 *gpos4 = nullptr; /* position buffer current when the graph was captured */
    int use_graphs = 1;            /* 0: launch every step's kernels eagerly */
    int fuse_step = 0;             /* 1: fused pair+leapfrog kernel where applicable */
    int cw_grid[2] = {0, 0};       /* blocks of the persistent list builder (single, batch) */
    int rebuild_coop = 1;          /* single systems: the rebuild as one cooperative kernel */
    unsigned long long dbg_bar_ns = 0; /* test hook: grid-barrier wait limit, ns (0: 50 ms) */
    int dbg_bar_drop = -1;         /* test hook: block of the cooperative rebuild that leaves
                                      before its first barrier (-1: none) */
    int coop_grid = 0;             /* its blocks (0: not found yet, -1: unavailable) */
    int nsm = 1;                   /* SMs of the device (found with cw_grid) */
    int rebuild_inline = 0;        /* step graphs: 1 = list passes inline (programmatic launches
                                      that return at once without a request), 0 = a conditional node */
    long long host_step = 0;       /* steps run so far (mirrors st->step) */
    std::vector<std::string> type_names;   /* element names per type (.fld), if known */
    double *io_dev = nullptr;      /* 4*pitch doubles for host transfers */
    int pair_tpa = 8;    /* threads per atom in the pair kernel */
    int pair_depth = 0;  /* list entries per lane and batch (0: the default for pair_tpa) */
    int centered = 0;    /* every position in [-L/2, L/2] (set at upload; the wraps keep it) */
    int list_tpa = 0;    /* list build: 0 = one warp per cell, else threads per atom */
    int fp64 = 0;        /* 1: force kernels in FP64 on the FP64 positions (md_set_precision) */
    double baro[3] = {1.0, 1000.0, 4.5e-5};   /* NPT: target bar, tau_p fs, compressibility 1/bar */
    md_p64 *p64_dev = nullptr;        /* FP64 model constants per replica (1 for a single system) */
    std::vector<float> rep_alfa;      /* damping alpha per replica of a batch */

    /* batches of replicas (md_create_batch; any number, 1 included) */
    int batch = 0;
    int nrep = 1;
    std::vector<md_rep> reps;
    std::vector<int> rep_natom;
    md_rep *reps_dev = nullptr;
    md_repstate *repst = nullptr;
    int *arep = nullptr;          /* atom -> replica (the same in both orders) */
    int *rep_upd = nullptr;       /* per replica: an atom moved >= skin/2 since its last build */
    int *crep = nullptr;          /* cell rank -> replica */
    float2 *ljr_dev = nullptr;    /* nrep x 64 (lj1, lj2) */
    unsigned long long *racc = nullptr; /* nrep x 3 fixed-point KE, PE, virial sums of a step */
    int2 *grid_tab = nullptr;     /* the MD_NGRID replica-aligned grids, concatenated */
    int grid_off[MD_NGRID] = {0}, grid_cnt[MD_NGRID] = {0};

    /* state at the start of an md_step call, kept on the device so that a
     * call whose list overflowed can be run again with a larger list */
    void *snap = nullptr;          /* one allocation holding every array below */
    size_t snap_bytes = 0;
    float4 *snap_p4 = nullptr, *snap_p4alt = nullptr;   /* the position buffers' roles */
    long long snap_host_step = 0;
    int overflow_retry = 1;        /* 0: report a list overflow inside md_step without re-running */
    int regrows = 0;               /* md_step calls re-run after a list overflow */
    int regrids = 0;               /* NPT: cell grids laid out again for changed boxes */
    md_pme pme;                    /* lkspace 2: the reciprocal Ewald sum (md_set_pme) */

    /* timing of the last md_step call (CUDA events on the stream) */
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

md_kparams md_make_kparams(const md_ctx *c);
/* 1 when a stencil cell's periodic image gives the reference's min-image
 * shift exactly: every candidate pair lies well inside half a box,
 * |d| <= (S+1) bin < 0.49 L on every axis. */
int md_cell_shift(const int stencil[3], const float binlen[3], const float box[3]);
/* Degrees of freedom of the temperature: 3N - 3 per system (integrator.cu:155). */
int md_ndf(const md_ctx *c);

/* Constants of the consistent potentials at the cutoff: the Coulomb shift
 * ucc (Wolf: erfc(a rc)/rc with A&S 7.1.26; reaction field: 1/rc + k rc^2/2),
 * rc^-6 and 1/rc, computed in FP64 and rounded once. */
inline void md_shift_consts(int lkspace, float rcutsq, float alfa, float reacf, float *ucc,
                            float *rc6i, float *rcinv)
{
    double rc = sqrt((double)rcutsq);
    *rcinv = (float)(1.0 / rc);
    *rc6i = (float)(1.0 / (rc * rc * rc * rc * rc * rc));
    if (lkspace == 1) {
        const double a1 = (double)0.254829592f, a2 = (double)-0.284496736f,
                     a3 = (double)1.421413741f, a4 = (double)-1.453152027f,
                     a5 = (double)1.061405429f;
        double x = (double)alfa * rc;
        double t = 1.0 / (1.0 + (double)0.3275911f * x);
        double poly = ((((a5 * t + a4) * t + a3) * t + a2) * t + a1);
        *ucc = (float)(poly * t * exp(-x * x) / rc);
    } else if (lkspace == 0) {
        *ucc = (float)(1.0 / rc + 0.5 * (double)reacf * rc * rc);
    } else {
        *ucc = 0.0f;
    }
}
/* ---- smooth particle-mesh Ewald (k_pme.cu) ---- */
/* grid K (all zero: off); lkspace 2 single systems only (md_set_pme checks) */
md_status pme_setup(md_ctx *c, const int K[3]);
void pme_free(md_ctx *c);
/* spread, FFTs, solve and gather of the reciprocal sum, added into the forces */
void launch_pme(md_ctx *c, const md_kparams &kp, bool energy);
/* Message returned by md_last_error(NULL, ...). */
void md_set_global_error(const std::string &msg);

/* ---- launchers (k_cells.cu) ---- */
void launch_check(md_ctx *c, const md_kparams &kp);
/* unconditional: build without looking at the device's rebuild request (the
 * body of a graph's conditional rebuild node, or a forced build).  In a
 * batch only the replicas whose atoms moved are rebuilt, unless
 * all_replicas is set (forced builds). */
void launch_rebuild(md_ctx *c, const md_kparams &kp, bool unconditional, bool all_replicas,
                    bool pdl = false);
void launch_set_condition(md_ctx *c, unsigned long long handle);
bool md_rebuild_coop(md_ctx *c);
/* ---- launchers (k_forces.cu) ---- */
void launch_forces(md_ctx *c, const md_kparams &kp, bool energy, int terms);
/* bonds and angles (when present and asked for in terms), added into the forces */
void launch_bonded(md_ctx *c, const md_kparams &kp, bool energy, int terms);
/* ---- launchers (k_pair64.cu): the FP64 mode ---- */
void launch_pair64(md_ctx *c, bool energy);
void launch_bonded64(md_ctx *c, bool energy, int has_bonds, int has_angles);
/* ---- launchers (k_integrate.cu) ---- */
/* cond / has_cond: graph condition (cudaGraphConditionalHandle) the kernel's
 * last block sets to "rebuild the list before the next force evaluation". */
void launch_leapfrog(md_ctx *c, const md_kparams &kp, int energy, unsigned long long cond,
                     int has_cond);
void launch_vv_first(md_ctx *c, const md_kparams &kp, unsigned long long cond, int has_cond);
void launch_vv_second(md_ctx *c, const md_kparams &kp, int energy);
void launch_thermo_from_state(md_ctx *c, const md_kparams &kp, int energy);
void launch_gather_out(md_ctx *c, const md_kparams &kp, int what, void *dst);
void launch_scatter_in(md_ctx *c, const md_kparams &kp, int what, const void *src);
/* ---- launchers (k_fused.cu) ---- */
/* Leapfrog systems without bonded terms step with one fused kernel. */
bool md_can_fuse(const md_ctx *c);
/* Pair forces + leapfrog + check in one kernel; swaps pos4 and pos4_alt. */
void launch_pair_leapfrog(md_ctx *c, const md_kparams &kp, unsigned long long cond, int has_cond);

/* ---- launchers of batches (k_batch.cu); the launchers above forward to
 * these for batch contexts (the list kernels of a batch live in k_cells.cu) ---- */
void launch_forces_b(md_ctx *c, const md_kparams &kp, bool energy, int terms);
void launch_leapfrog_b(md_ctx *c, const md_kparams &kp, int energy, unsigned long long cond,
                       int has_cond);
void launch_vv_first_b(md_ctx *c, const md_kparams &kp, unsigned long long cond, int has_cond);
void launch_vv_second_b(md_ctx *c, const md_kparams &kp, int energy, int kick);
/* NPT: every replica's box and cell geometry scaled by the factor its last
 * step applied to its positions (after each leapfrog step of an NPT batch) */
void launch_npt_box_b(md_ctx *c);

/* List entries each pair-kernel lane loads per batch for the context's
 * lanes per atom: the autotuner's choice, else the default (TPA * depth
 * divides the 32-entry row quantum). */
inline int md_pair_depth(const md_ctx *c)
{
    const int t = c->pair_tpa;
    if (c->pair_depth > 0 && MD_LIST_QUANTUM % (t * c->pair_depth) == 0) return c->pair_depth;
    return t >= 32 ? 1 : (t >= 16 ? 2 : (t >= 8 ? 4 : 8));
}

/* Launches kernel k so that it may start before its predecessor in the
 * stream ends (the kernel must call pdl_wait() before touching data that
 * predecessor writes). */
template <typename... KArgs, typename... Args>
inline cudaError_t md_launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, cudaStream_t s,
                                 Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

#define MD_CUDA_TRY(c, expr)                                                   \
    do {                                                                       \
        cudaError_t e_ = (expr);                                               \
        if (e_ != cudaSuccess) {                                               \
            (c)->last_error = std::string(#expr) + ": " + cudaGetErrorString(e_); \
            return MD_ERR_CUDA;                                                \
        }                                                                      \
    } while (0)

#endif
