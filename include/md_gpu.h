/*
 * md_gpu.h -- C ABI of libmdgpu_gb300: md_gpu's per-step force-and-integrate
 * path (neighbour list, LJ + Wolf / reaction-field pair forces, harmonic
 * bonds and angles, leapfrog / Berendsen / velocity-Verlet / Nose-Hoover
 * integrators) as hand-written sm_103a kernels.
 *
 * Plain C types only.  Every call returns an md_status (the reference exits
 * the process on any CUDA error, gpu_properties.cu:75-81).  One md_ctx per
 * system; distinct contexts may be used from distinct host threads.  Unless
 * stated otherwise host arrays are in the original atom order of the input.
 *
 * Units as in the reference: A, fs, g/mol, kJ/mol, e.  Masses in the
 * descriptor are g/mol * 1e4, the reference's stored unit (simulation.cu:177).
 */
#ifndef MD_GPU_H
#define MD_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct md_ctx md_ctx;

typedef enum {
    MD_OK = 0,
    MD_ERR_ARG = 1,            /* invalid argument */
    MD_ERR_IO = 2,             /* file cannot be opened */
    MD_ERR_PARSE = 3,          /* input file does not follow the grammar */
    MD_ERR_CUDA = 4,           /* CUDA runtime error (see md_last_error) */
    MD_ERR_LIST_OVERFLOW = 5,  /* an atom has more neighbours than the list holds */
    MD_ERR_BONDED = 6,         /* more than four bonds / angles on one atom */
    MD_ERR_UNSUPPORTED = 7,    /* option not implemented */
    MD_ERR_BOX = 8             /* cutoff + skin larger than half the box */
} md_status;

/* Integrators.  LEAPFROG follows nve_leapfrog.cu / nvt_leapfrog_ber.cu (the
 * reference's active path, runGPU.cu:71); VV is velocity Verlet NVE with the
 * half kick counted once (nve_vverlet.cu:49 adds it twice); NH is velocity
 * Verlet with one Nose-Hoover thermostat (nvt_vverlet_nh.cu has no such
 * implementation: it is a copy of the Berendsen file). */
typedef enum { MD_LEAPFROG = 0, MD_VV = 1, MD_NH = 2 } md_integrator;

/* Force terms for md_compute_forces (bit mask). */
/* MD_TERM_RECIP: the reciprocal Ewald sum of md_set_pme (with its self,
 * background and exclusion terms); no counterpart in the reference, whose
 * lkspace 2 computes the real-space term only */
enum { MD_TERM_PAIR = 1, MD_TERM_BOND = 2, MD_TERM_ANGLE = 4, MD_TERM_RECIP = 8, MD_TERM_ALL = 15 };

/* A system as the reference holds it after SimulationInit (simulation.h:51-122). */
typedef struct {
    int natom;
    int ntype;                  /* <= 8 (forces.cu:48-49) */
    float box[3];               /* box edge, A; coordinates centred in [-L/2, L/2] (others are
                                   taken, on slower list and pair paths: md_info) */
    const int *itype;           /* natom, 0-based */
    const float *charge;        /* natom, e */
    const float *pos;           /* 3*natom */
    const float *vel;           /* 3*natom, A/fs (may be NULL: zero) */
    const float *type_mass;     /* ntype, g/mol * 1e4 */
    const float *lj1;           /* ntype*ntype (row stride ntype): 48 eps sig^12 or 12 A */
    const float *lj2;           /* ntype*ntype: 24 eps sig^6 or 6 B */
    int nbonds;
    const int *bonds;           /* 3*nbonds: type, i, j (0-based) */
    const float *bnd1, *bnd2;   /* per bond type: 2k, r0 */
    int nangle;
    const int *angles;          /* 4*nangle: type, i, j (centre), k (0-based) */
    const float *ang1, *ang2;   /* per angle type: 2k, theta0 (rad) */
    /* run parameters (params / integr, simulation.h:88-122) */
    int lkspace;                /* 0 reaction field, 1 Wolf, 2 Ewald real space (alpha only;
                                   md_set_pme adds the reciprocal sum) */
    float rcutsq;               /* squared cutoff, A^2 */
    float reacf;                /* 2(eps-1)/(2eps+1)/rc^3 (lkspace 0) */
    float alfa;                 /* damping alpha, 1/A (lkspace 1, 2) */
    float skin;                 /* list skin, A */
    int nmaxlist;               /* list capacity per atom (minimum) */
    int enstype;                /* 0 NVE, 1 NVT, 2 NPT (Berendsen leapfrog; md_create makes
                                   the context a batch of one replica, see md_set_barostat) */
    float temper_0;             /* K */
    float dt;                   /* fs */
    float tau_t;                /* thermostat time constant, fs (Berendsen and NH) */
    int integrator;             /* md_integrator */
} md_system_desc;

/* Thermodynamic record of one step (FP64 reductions on the device). */
typedef struct {
    long long step;
    double ke;           /* kJ/mol */
    double temper;       /* K, 2 KE / ((3N-3) R) */
    double pe;           /* kJ/mol, consistent potential (when computed, else 0) */
    double virial;       /* sum over pairs of F.r / ... : sum ff r^2 / 6 (when computed) */
    double conserved;    /* KE + PE (+ NH terms) (when PE computed) */
    double xi;           /* NH thermostat variable, 1/fs */
    double lambda;       /* Berendsen scale of the step */
    int builds;          /* neighbour-list builds so far */
    int flags;           /* bit 0: energies computed this step */
} md_thermo;

const char *md_status_string(md_status s);
/* Copies the last error message of ctx (may be NULL for global errors). */
md_status md_last_error(const md_ctx *ctx, char *buf, int len);

/* Many independent systems ("replicas", e.g. uneven sizes and per-replica
 * force fields) in one context, advanced together: every stage of a step is
 * one launch over all replicas, and md_step replays one captured graph for
 * the whole batch.  No counterpart in the reference, which runs one system
 * per process.  descs[r] describes replica r exactly as md_create would take
 * it; replicas must share lkspace, integrator, enstype, dt and tau_t, and
 * the replicas that have bonds (angles) must share the bonded parameter
 * tables bnd1/bnd2 (ang1/ang2) (MD_ERR_ARG otherwise).  Box, cutoff, skin,
 * alpha, LJ table, masses, charges, temperature, bonds and angles are per
 * replica.  Host arrays of
 * the context (positions, velocities, forces, energies, neighbour lists,
 * order) hold the replicas' atoms concatenated in replica order; the
 * neighbour list of a replica holds only its own atoms.  md_get_thermo
 * returns the batch totals (temperature over all degrees of freedom);
 * md_get_replica_thermo the per-replica values.  A batch of one replica is
 * a batch context (the adjoint, md_adjoint_run, takes batch contexts). */
md_status md_create_batch(const md_system_desc *descs, int nrep, void *stream, md_ctx **out);
/* Per-replica state after the last step of a batch (out[r], r < nrep and
 * < the batch's replica count; synchronises the stream). */
md_status md_get_replica_thermo(md_ctx *ctx, md_thermo *out, int nrep);

/* Differentiable trajectories (no counterpart in the reference).  For a
 * batch context with velocity Verlet NVE, md_adjoint_run runs nsteps steps
 * from the current state and evaluates per replica the loss
 *   L = w_pe <U>/N + w_rdf sum_b (gbar_b - target_b)^2,
 * <U> the average potential energy over the nsteps + 1 frames, gbar the
 * frame average of the Na-Cl-style RDF of atom types (rdf_a, rdf_b) smoothed
 * by Gaussians of width rdf_sigma on nbins bins of width rdf_dr (centres at
 * (b + 1/2) rdf_dr; the range plus 5 sigma must lie inside every replica's
 * cutoff).  With gradient != 0 it also returns dL/d lj1[a][b] and
 * dL/d lj2[a][b] (8x8 per replica, entry a*8+b as used by atoms of type a;
 * the derivative for a symmetric pair parameter is the sum of the (a,b) and
 * (b,a) entries) and dL/d ln s for a common charge scale s, by the discrete
 * adjoint of the integrator with (x, v) checkpoints every `checkpoint` steps
 * and recompute.  The context is left at the end of the trajectory.
 * target: nrep*nbins (NULL = 0); loss: nrep; gbar: nrep*nbins (may be NULL);
 * dlj1, dlj2: nrep*64; dlns: nrep. */
typedef struct {
    int nsteps;         /* steps of the trajectory (frames 0..nsteps) */
    int checkpoint;     /* steps between checkpoints (recompute segment) */
    int gradient;       /* 0: forward pass only (loss, gbar) */
    double w_pe, w_rdf; /* loss weights */
    int rdf_a, rdf_b;   /* atom types of the RDF pair (0-based) */
    int nbins;          /* <= 256 */
    double rdf_dr, rdf_sigma;   /* A */
} md_adjoint_cfg;
md_status md_adjoint_run(md_ctx *ctx, const md_adjoint_cfg *cfg, const double *target, double *loss,
                         double *gbar, double *dlj1, double *dlj2, double *dlns);

/* SimulationInit + config_init + forces_init + neighborlist_init +
 * integrate_init (simulation.cu:40, runGPU.cu:53-60): reads <base>.inp,
 * <base>.fld and <base>.cfg in the reference grammar, uploads the system
 * and builds the first neighbour list.  stream: cudaStream_t or NULL. */
md_status md_create_from_files(const char *base, void *stream, md_ctx **out);
/* The same from arrays (no files). */
md_status md_create(const md_system_desc *desc, void *stream, md_ctx **out);
/* forces_finish + config_finish + integrate_finish + neighborlist_finish
 * (runGPU.cu:107-113). */
md_status md_destroy(md_ctx *ctx);

/* config_HostToDevice / config_DeviceToHost (config.cu:56-77), original order. */
md_status md_set_positions(md_ctx *ctx, const double *pos3);
md_status md_set_velocities(md_ctx *ctx, const double *vel3);
md_status md_get_positions(md_ctx *ctx, double *pos3);
md_status md_get_velocities(md_ctx *ctx, double *vel3);
/* Forces of the last force evaluation: fx, fy, fz, sum ff r^2 per atom
 * (the reference's float4 force record, pair_forces.cu:117-120). */
md_status md_get_forces(md_ctx *ctx, double *force4);
/* Per-atom potential energy of the last energy evaluation (half of each pair). */
md_status md_get_energies(md_ctx *ctx, double *epot);

/* neighborlist() (neighborlist.cu:109-146) without the host round trip:
 * force = 1 rebuilds unconditionally, 0 only if an atom moved >= skin/2. */
md_status md_update_neighbors(md_ctx *ctx, int force);
/* The current list in the reference's layout (neighborlist.cu:284):
 * nnlist[i + pitch*k] = j (original indices, ascending), nnlist_max[i].
 * nnlist holds pitch*nmax entries; returns MD_ERR_LIST_OVERFLOW if any
 * atom has more than nmax neighbours. */
md_status md_get_neighbor_list(md_ctx *ctx, unsigned *nnlist, unsigned *nnlist_max, int pitch,
                               int nmax);

/* forces() + energy() (forces.cu:189-231): pair, bond and angle terms
 * selected by `terms`; energy != 0 also computes per-atom potential energy
 * and the virial (FP64 totals, see md_get_thermo). */
md_status md_compute_forces(md_ctx *ctx, int terms, int energy);

/* nsteps iterations of the reference's loop body (runGPU.cu:69-104):
 * list check and rebuild, forces, integrate.  energy_every > 0 computes
 * energies on steps that are multiples of it (the reference's timprn).
 * Steps run as a captured CUDA graph; no host synchronisation inside.  A
 * list rebuild inside the run that finds a row longer than the list holds
 * (the reference writes past its list then, neighborlist.cu:284) truncates
 * rows, so the call saves the state on the device when it starts; after an
 * overflow it restores that state, grows the list, rebuilds it and runs the
 * same steps again (md_info.list_regrows counts such calls), and returns
 * MD_ERR_LIST_OVERFLOW only when that fails three times. */
md_status md_step(md_ctx *ctx, int nsteps, int energy_every);
/* The integrate phase of one step alone, with the forces of the last
 * md_compute_forces (for callers that drive the phases themselves, as the
 * reference's loop does).  md_integrate = integrate() (integrator.cu:131-173:
 * leapfrog, Berendsen when the ensemble is NVT); energy != 0 puts the
 * energies of that force evaluation in the step's record.  md_integrate_pre /
 * md_integrate_cor = integrate_pre() / integrate_cor() (integrator.h:53-54):
 * the two halves of velocity Verlet around the force evaluation (standard VV,
 * and Nose-Hoover for NVT); the first md_integrate_pre turns a leapfrog
 * context into a velocity-Verlet one.  Each synchronises the stream. */
md_status md_integrate(md_ctx *ctx, int energy);
md_status md_integrate_pre(md_ctx *ctx);
md_status md_integrate_cor(md_ctx *ctx, int energy);
/* Record of the most recent step (synchronises the stream). */
md_status md_get_thermo(md_ctx *ctx, md_thermo *out);
/* The last min(n, nsteps run) records, oldest first; returns the count in *got. */
md_status md_get_thermo_history(md_ctx *ctx, md_thermo *out, int n, int *got);

/* Per-replica records of a batch (no counterpart in the reference): for the
 * last min(n, steps run, 4096) steps, oldest first, out[(t * nrep + r) * 3 +
 * {0, 1, 2}] = replica r's kinetic energy, potential energy and conserved
 * quantity (KE + PE, plus the Nose-Hoover terms) after step t, kJ/mol; PE
 * and the conserved quantity are 0 on steps without energies (md_step's
 * energy_every).  The matching batch records are md_get_thermo_history's.
 * *got = the number of steps returned.  MD_ERR_ARG for a single system. */
md_status md_get_replica_history(md_ctx *ctx, double *out, int n, int *got);

/* One call end to end from host buffers: uploads pos/vel (3N doubles),
 * runs nsteps, downloads pos/vel and the per-step records (nsteps). */
md_status md_run_host(md_ctx *ctx, double *pos3, double *vel3, int nsteps, int energy_every,
                      md_thermo *records);

/* Current configuration in the reference's .cfg grammar (simulation.cu:331-339),
 * with full float precision. */
md_status md_write_cfg(md_ctx *ctx, const char *path);
/* One frame in XYZ format (the reference's ConfigFinish writes one, with %f,
 * simulation.cu:323-328): atom count, a comment line with the step and box,
 * then "name x y z" per atom in original order with full double precision
 * (names from the .fld when the context was read from files, else T1, T2,
 * ...).  append != 0 adds the frame at the end of the file: a trajectory. */
md_status md_write_xyz(md_ctx *ctx, const char *path, int append);
/* Restart (no counterpart in the reference): md_write_restart stores the
 * state of a single system exactly (FP64 positions and velocities as
 * stored, the step count, the thermostat state and the last step's record);
 * md_read_restart loads it
 * into a context of the same system (same atom count), rebuilds the list
 * and continues from there.  Binary, native byte order. */
md_status md_write_restart(md_ctx *ctx, const char *path);
md_status md_read_restart(md_ctx *ctx, const char *path);

/* Introspection for tests and tools. */
typedef struct {
    int natom, pitch, capacity, ncell[3], stencil[3];
    float binlen[3];
    int pair_threads_per_atom, list_threads_per_atom;
    int builds;
    int max_neighbors;
    int kernels_per_step;   /* kernel launches of one step of a step graph without a rebuild
                               (inline rebuild passes included: they run every step) */
    int kernels_per_rebuild; /* kernels a list rebuild adds to a step (0 with inline passes) */
    int kernels_per_graph;  /* kernels a step graph runs besides its steps (condition set-up) */
    int pair_entries_per_lane; /* list entries each pair-kernel lane loads per batch */
    int positions_centered; /* 1: every position uploaded last lay in [-L/2, L/2] per axis,
                               so the fast paths that rely on it are on (the integrators
                               keep it so); 0: cells bin periodic images, every pair
                               takes the minimum-image shift */
    int fused_step;         /* 1: step graphs run pair forces and update as one kernel */
    int rebuild_inline;     /* 1: step graphs hold the rebuild passes inline, 0: behind a
                               conditional node */
    int list_regrows;       /* md_step calls run again after their list overflowed (md_step) */
    int cell_regrids;       /* NPT batches: cell grids laid out again for a changed box (md_step) */
    int pme_grid[3];        /* md_set_pme grid points per axis (0: no reciprocal sum) */
} md_info;
md_status md_get_info(md_ctx *ctx, md_info *out);
/* Sorted -> original index map of the current atom order. */
md_status md_get_order(md_ctx *ctx, int *perm);
/* Hilbert rank of every cell (linear index x + nx*(y + ny*z)). */
md_status md_get_cell_ranks(md_ctx *ctx, int *rank);
/* Tuning knobs: threads per atom of the pair kernel (1, 2, 4, 8, 16, 32) and
 * the list builder (0 = one warp per cell, the default; or 1..32 threads per
 * atom; batches take 0 only).  Every setting builds the identical list. */
md_status md_set_tuning(md_ctx *ctx, int pair_tpa, int list_tpa);
/* List entries each pair-kernel lane loads per batch (memory-level
 * parallelism against registers): 0 = the default for the lane count (8 for
 * 1-4 lanes, 4 for 8, 2 for 16, 1 for 32); also half the default at 4, 8
 * and 16 lanes.  md_set_tuning resets it to 0. */
md_status md_set_pair_depth(md_ctx *ctx, int depth);
/* Autotuner: times the pair kernel for 2/4/8/16 threads per atom (also at
 * 4/8/16 threads with half the default entries per lane and batch) and the
 * list builders (warp per cell, 4/8/16 threads per atom) on the
 * current state and keeps the fastest of each; returns the choice.  It also
 * times the step graphs by running steps: fused or separate pair and
 * integrator kernels (leapfrog systems without bonded terms), and for single
 * systems the rebuild inline or behind a conditional node
 * (md_set_graph_rebuild), each for the three fastest pair settings.  The
 * system advances 128 steps per combination tried (up to 12; batches have
 * one and do not advance). */
md_status md_autotune(md_ctx *ctx, int *pair_tpa, int *list_tpa);
/* Per-type exclusions (no counterpart in the reference, which excludes only
 * 1-2 bonded pairs): bit b of mask[a] excludes every pair of types a and b
 * from the neighbour list (made symmetric); ntype entries.  Rebuilds the list. */
md_status md_set_type_exclusions(md_ctx *ctx, const unsigned *mask);
/* Arithmetic of the force kernels: 32 (the default) evaluates pair terms in
 * FP32 on the FP32 copy of the positions, as the reference's kernels do
 * (pair_forces.cu:34-205); 64 evaluates pair, bond and angle terms in FP64
 * on the FP64 positions with IEEE sqrt, divide, exp and log (the plain FP64
 * form of the same force law, A&S erfc included).  Forces, integrators and
 * reductions are shared (int64 fixed-point forces, FP64 state).  No
 * counterpart in the reference; the FP64 mode is the GPU reference point of
 * the precision checks.  Recomputes the forces of the current state.  FP64
 * contexts run no fused step and no adjoint (md_adjoint_run returns
 * MD_ERR_UNSUPPORTED). */
md_status md_set_precision(md_ctx *ctx, int bits);
/* NPT: the Berendsen barostat the reference sketches (npt_leapfrog_ber.cu:
 * 28-125 sums the kinetic energy and virial of a leapfrog step but never
 * changes the box, and integrator.cu:157-164 leaves it uncalled).  Each step
 * of a leapfrog NPT context (enstype 2: Berendsen thermostat as in NVT)
 * computes every replica's pressure P = (2 KE + sum over pairs of F.r) /
 * (3 V) from its kinetic energy and virial, and the next step scales the
 * replica's positions and box by mu = 1 - beta dt / (3 tau_p) (P0 - P)
 * (|mu - 1| <= 1e-4 per step), on the device.  press_bar = P0 in bar (the
 * .inp's npt line), tau_p_fs (default 1000; ".inp" extension line
 * "tau_p: <fs>"), compressibility_per_bar = beta (default 4.5e-5;
 * "compressibility: <1/bar>").  The cell grid is laid out 3% longer than
 * the list needs; md_step runs NPT batches in chunks of at most 128 steps
 * (whole multiples of energy_every) and, between chunks, lays the cells
 * out again (and rebuilds the lists) for every replica whose cells have
 * shrunk by half that margin or whose box has room for one more cell
 * (md_info.cell_regrids counts these).  MD_ERR_BOX remains for a box that
 * shrinks past the margin inside one step graph or below twice the list
 * radius.  Bonds add their virial, angles none (as the reference's
 * angle_forces). */
md_status md_set_barostat(md_ctx *ctx, double press_bar, double tau_p_fs, double compressibility_per_bar);
/* Long-range electrostatics for lkspace 2 ("Ewald": the reference reads
 * kmax but computes the real-space term only, simulation.cu:91-95,
 * forces.cu:97-113; its k-space code is an unbuilt copy of GROMACS's
 * pme.c): adds the reciprocal Ewald sum by smooth particle-mesh Ewald with
 * cubic B-splines on a k0 x k1 x k2 grid (multiples of 8 in [16, 2048];
 * all zero: off, the reference's behaviour), the self term
 * -qfac alpha/sqrt(pi) sum q^2, the background of a net charge, and the
 * removal of each atom's excluded partners' erf(alpha r)/r term.  Forces are
 * added into the fixed-point forces in every force evaluation (md_step,
 * md_compute_forces with MD_TERM_RECIP), energies into the per-atom
 * energies.  Single systems only, FP32 mode, no type exclusions.  An .inp
 * extension line "pme_spacing: <A>" sets the smallest such grid with at
 * most that spacing.  No counterpart in the reference. */
md_status md_set_pme(md_ctx *ctx, int k0, int k1, int k2);
/* Box edges (nrep x 3, A) and last-step pressure (nrep, bar; may be NULL)
 * of the replicas of a batch after the last md_step (NPT moves them); for a
 * single system its fixed box and pressure 0.  Synchronises the stream. */
md_status md_get_replica_box(md_ctx *ctx, double *box3, double *pressure_bar, int nrep);
/* Test hook of the one-kernel list rebuild of a single system (no
 * counterpart in the reference, whose list build has no grid barriers):
 * its phases are separated by grid barriers whose waits give up after
 * timeout_ms (0: the default, 50 ms) and set a sticky error; with
 * drop_block >= 0 that block of the rebuild leaves before the first barrier,
 * so the other blocks' waits run out.  After a timed-out wait every block
 * of the rebuild returns at once and every later launch of the rebuild
 * returns without work; the step kernels run on with the list and atom
 * order as the interrupted rebuild left them (every index still in range),
 * and the next synchronising call (md_step, md_update_neighbors, ...)
 * returns MD_ERR_CUDA with the message "a grid barrier of the list rebuild
 * timed out".  The context must then be destroyed (its atom order may be
 * half permuted); the CUDA context stays usable.  timeout_ms = 0 and drop_block = -1 restore the defaults. */
md_status md_debug_rebuild_barrier(md_ctx *ctx, double timeout_ms, int drop_block);
/* Test hook (no counterpart in the reference): gives the list capacity
 * entries per atom (a multiple of 32, >= 32; the list is reallocated) and
 * makes the next step rebuild it, so that a too-small list overflows inside
 * a run; retry 0 makes md_step report the overflow (MD_ERR_LIST_OVERFLOW)
 * instead of growing the list and running the steps again. */
md_status md_debug_list_capacity(md_ctx *ctx, int capacity, int retry);
/* md_step launches each step's kernels eagerly instead of replaying a
 * captured graph when use_graphs is 0 (for profilers and debugging). */
md_status md_set_graphs(md_ctx *ctx, int use_graphs);
/* Leapfrog systems without bonded terms: 1 runs each step (pair forces and
 * the leapfrog update) as one kernel, 0 as two; MD_ERR_UNSUPPORTED for other
 * systems when asked for 1.  md_autotune times both and keeps the faster. */
md_status md_set_fused_step(md_ctx *ctx, int fused);
/* How a step graph holds the neighbour-list rebuild (single systems): 0 (the
 * default) a conditional node per step whose body is the rebuild; 1 the
 * rebuild passes inline in every step, launched as programmatic dependents
 * that return at once when no rebuild is due.  Both rebuild at the same
 * steps and give the same trajectory; md_autotune keeps the faster. */
md_status md_set_graph_rebuild(md_ctx *ctx, int inline_passes);
/* Milliseconds of device time of the last md_step call (CUDA events). */
md_status md_last_step_ms(md_ctx *ctx, float *ms);
/* The pair-force kernel alone, nrep launches on the context's stream between
 * CUDA events: average milliseconds per launch (the force arrays are
 * recomputed afterwards, so the state is unchanged). */
md_status md_time_pair(md_ctx *ctx, int nrep, float *ms_per_launch);
/* A full list build (binning, Hilbert sort, permutation, list), nrep times
 * between CUDA events on the context's stream: average milliseconds. */
md_status md_time_rebuild(md_ctx *ctx, int nrep, float *ms_per_build);
/* FP32 FMA throughput of the current device (TFLOP/s, best of 5): the
 * measured FP32-pipe peak the pair kernel is compared against. */
md_status md_probe_fp32_peak(double *tflops);

/* Kinetic energy and temperature of a float4 velocity array, one record per
 * atom holding (vx, vy, vz, mass * 1e4), without allocating any device
 * memory.  No counterpart in the reference: it
 * serves callers that cannot let a library call cudaMalloc, such as hosts that
 * manage all device memory through their own allocator and budget, or step
 * loops that must not risk the device synchronisation cudaMalloc/cudaFree can
 * cause.  vel4 and out are device pointers supplied by the caller; out[0] =
 * KE (kJ/mol, FP64 fixed-order sum), out[1] = T = 2 KE / ((3N-3) R).  Scratch
 * is a fixed 32 KB __device__ array shared by all calls: at most 1,048,576
 * atoms (larger calls return MD_ERR_ARG), and calls that overlap on the GPU
 * race.  A call made outside stream capture resolves the array's address on
 * the current device (so a device reset between calls is harmless); a call
 * made while its stream is being captured reuses the address the last
 * uncaptured call on that device resolved, so make one call on each device
 * before capturing.  stream: cudaStream_t or NULL. */
md_status md_ref_kinetic_energy_noalloc(const void *vel4, int natom, double *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
