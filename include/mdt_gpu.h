/*
 * mdt_gpu.h -- C ABI of the md_tian2 GB300 force-and-propagation engine (libmdt_gpu.so).
 *
 * The reference (maurergroup/md_tian2) exposes its hot path as Fortran module
 * procedures operating on one `type(universe)`.  This library replaces that path for a
 * BATCH of independent trajectories on one GPU.  Every entry point:
 *   - returns int32_t status: 0 = MDT_OK, negative = error (never aborts the process;
 *     the reference's `print + stop` becomes an error code + mdt_last_error text);
 *   - takes plain pointers and sizes; host arrays use the reference's Fortran order,
 *     i.e. per trajectory r(3, nbeads, natoms) with the x/y/z index fastest, and the
 *     trajectories concatenated;
 *   - is callable from Fortran through iso_c_binding (include/mdt_gpu.f90).
 * Threading: one context per host thread; calls on one context are serialised on the
 * context's CUDA stream.  The caller owns host memory, the library owns device memory.
 */
#ifndef MDT_GPU_H
#define MDT_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MDT_OK 0
#define MDT_ERR_ARG -1         /* invalid argument (the reference would `stop`) */
#define MDT_ERR_CUDA -2        /* CUDA runtime error */
#define MDT_ERR_STATE -3       /* call order violated (e.g. no batch defined) */
#define MDT_ERR_UNSUPPORTED -4 /* configuration outside what this engine implements */
#define MDT_ERR_NOMEM -5       /* device allocation failed */
#define MDT_ERR_TOO_LARGE -6   /* configuration beyond a fixed maximum size */

/* ids shared with the reference, src/constants.f90:64-71,107-115 */
#define MDT_PES_EMT 2003
#define MDT_PES_NENE 2008
#define MDT_PES_SURROGATE 2100 /* ACSF->MLP surrogate of EMT with EMT fallback; no reference id */
#define MDT_PROP_VERLET 1001
#define MDT_PROP_LANGEVIN 1003       /* LDFA friction from the EMT density */
#define MDT_PROP_ANDERSEN 1005
#define MDT_PROP_PILE 1006
#define MDT_PROP_LANGEVIN_CONST 1007 /* constant friction; no reference counterpart */
#define MDT_ENERGY_AND_FORCE 3001
#define MDT_ENERGY_ONLY 3002

/* force arithmetic */
#define MDT_PREC_FP64 0
#define MDT_PREC_FP32 1
#define MDT_PREC_BF16 2 /* FP32 descriptors and forces, network GEMMs on the tensor cores with
                           BF16 operands and FP32 accumulation: fused in the thread-per-atom
                           kernel of radial-only networks (forces and MD steps); for other
                           MDT_PES_NENE networks (<= 2 elements, <= 2 hidden layers of <= 32
                           nodes, <= 48 descriptors) mdt_calc_force runs the network as a pass
                           of its own between the FP32 descriptor and force passes; no
                           counterpart in the reference */
#define MDT_PREC_BF16X3 3 /* as MDT_PREC_BF16 with every operand split in a BF16 high and low
                             part, three MMAs per K step (about 16 significant bits) */

/* trajectory status (mdt_traj_summary.status) */
#define MDT_TRAJ_RUNNING 0
#define MDT_TRAJ_EXIT_UPPER 1   /* projectile above pul, md_tian2.f90:88-89 */
#define MDT_TRAJ_EXIT_LOWER 2   /* projectile below pll, md_tian2.f90:91-92 */
#define MDT_TRAJ_STEP_LIMIT 3   /* the step limit (nsteps) was reached, md_tian2.f90:78 */
#define MDT_TRAJ_ERR_DENSITY -10 /* negative EMT density in ldfa, md_algo.f90:551-554 */
#define MDT_TRAJ_ERR_NONFINITE -11 /* a position or velocity stopped being finite (fused MD
                                      steps only; the reference has no such check) */

typedef struct mdt_ctx mdt_ctx;

/* Propagation parameters: the simparams fields the hot path reads
   (src/run_config.f90:34-85). */
typedef struct mdt_prop_params {
    double step;          /* fs */
    double Tsurf, Tproj;  /* K */
    double pile_tau;      /* fs, default 200 (run_config.f90:120) */
    double andersen_time; /* fs, default 30 (run_config.f90:119) */
    double gamma_const;   /* 1/fs, MDT_PROP_LANGEVIN_CONST only */
    double pul, pll;      /* projectile exit limits, A */
    uint64_t seed;        /* counter-based RNG key; each trajectory adds its index */
    int32_t use_exit;     /* 1: stop a trajectory when its projectile passes pul/pll */
    int32_t rng_mode;     /* 0: on-device Philox; 1: arrays from mdt_set_random_arrays */
} mdt_prop_params;

typedef struct mdt_traj_summary {
    int32_t status;       /* MDT_TRAJ_* */
    int32_t steps_done;
    double epot;          /* mean bead potential energy, eV */
    double ekin_p, ekin_l;/* atom_ekin, universe_mod.f90:433-458 */
    double ebead;         /* ring-polymer spring energy, rpmd.f90:244-267 */
} mdt_traj_summary;

/* ---- context ------------------------------------------------------------- */
int32_t mdt_create(int32_t device, mdt_ctx **out);
int32_t mdt_destroy(mdt_ctx *ctx);
const char *mdt_last_error(const mdt_ctx *ctx);
int32_t mdt_synchronize(mdt_ctx *ctx);
/* use an existing cudaStream_t (0 = the context's own stream) */
int32_t mdt_set_stream(mdt_ctx *ctx, void *cuda_stream);

/* ---- PES parameters --------------------------------------------------------
 * Replaces read_emt (src/pes_emt_mod.f90:49-190): per-type EMT parameters
 * (eta2 [1/A], n0 [1/A^3], E0 [eV], lambda [1/A], V0 [eV], kappa [1/A], s0 [A]) and
 * the (ntypes x ntypes) column-major pes table (MDT_PES_EMT where EMT acts). */
int32_t mdt_emt_set_params(mdt_ctx *ctx, int32_t ntypes, const double *eta2, const double *n0,
                           const double *e0, const double *lambda, const double *v0, const double *kappa,
                           const double *s0, const int32_t *pes);

/* HDNNP model: what read_nene (src/pes_nene_mod.f90:123-5759) extracts from input.nn,
   scaling.data and weights.XXX.data.  Arrays per element e (ascending nuclear charge) and
   symmetry function s (RuNNer's canonical order, RuNNer_src/sortsymfunctions.f90) at
   [e*maxsf + s]; lengths in bohr, energies in Hartree, as inside RuNNer.  Supported
   subset: symmetry-function types 2 and 3 with one cutoff radius per element, cutoff
   types 0-8, activations t g l c s S e p h, at most 4 elements, 64 symmetry functions,
   4 layers of 64 nodes. */
typedef struct mdt_nn_model {
    int32_t nelem;
    const int32_t *z;          /* nuclear charge per element */
    int32_t maxsf;
    const int32_t *nsf;        /* symmetry functions per element */
    const int32_t *sftype;     /* 2 (radial) or 3 (angular) */
    const double *eta, *rshift, *lambda, *zeta, *rc;
    const int32_t *e1, *e2;    /* neighbour nuclear charges */
    const double *smin, *smax, *savg;  /* scaling.data columns */
    int32_t scalesym, centersym;
    double scmin, scmax;
    int32_t cutoff_type;
    double cutoff_alpha;
    int32_t nlayers;           /* hidden + output layers */
    int32_t maxnodes;
    const int32_t *nodes;      /* per element nlayers+1 entries, nodes[0] = nsf */
    const uint8_t *act;        /* per element nlayers*maxnodes activation letters */
    int32_t maxweights;
    const double *weights;     /* per element maxweights, calconenn order */
    int32_t normnodes;
    int32_t remove_atom_energies;
    const double *atom_energy; /* Ha per element */
} mdt_nn_model;

/* Replaces read_nene: install an HDNNP.  z_of_type[ntypes] gives the nuclear charge of
   each universe type (0: type not handled by the network); max_neighbors bounds the
   per-atom neighbour list (0 = 192). */
int32_t mdt_nn_set_model(mdt_ctx *ctx, const mdt_nn_model *model, int32_t ntypes, const int32_t *z_of_type,
                         int32_t max_neighbors);

/* Select the potential used by mdt_calc_force / mdt_md_steps: MDT_PES_EMT, MDT_PES_NENE
   or MDT_PES_SURROGATE (network forces; a bead whose symmetry functions leave
   [min - margin*(max-min), max + margin*(max-min)] is evaluated with FP64 EMT instead). */
int32_t mdt_set_pes(mdt_ctx *ctx, int32_t pes_kind, double range_margin);

/* FP32 network evaluations use a dedicated fast kernel when the model qualifies (G2 and
   narrow G3 only, one cosine cutoff shared by all functions, G3 of each element over one
   neighbour-element pair with lambda = +-1 and zeta in {1, 4, 16}, at most 4 G3 eta
   values, max_neighbors <= 255); results equal the generic kernels within FP32
   rounding.  enable = 0 forces the generic kernels.  Returns 1 if the installed model
   qualifies, else 0 (no replacement in the reference: RuNNer has one code path). */
int32_t mdt_nn_fast_path(mdt_ctx *ctx, int32_t enable);

/* Within the fast path, radial-only models (every function a G2 under one cosine cutoff,
   at most two elements with the same (eta, r_s) list per neighbour element, one or two
   hidden layers of at most 32 nodes, one activation per layer) run on a thread-per-atom
   kernel when the batch has single-bead trajectories of at most 512 atoms (and, for
   mdt_md_steps, Verlet or constant-friction Langevin propagators).  enable = 0 keeps
   them on the warp-per-atom fast kernel.  Returns 1 if the installed model qualifies,
   else 0 (no replacement in the reference: src/pes_nene_mod.f90:7145 has one path). */
int32_t mdt_nn_radial_kernel(mdt_ctx *ctx, int32_t enable);

/* Largest CTA (atoms of the trajectories packed into one CTA, 32..512, default 512) the
   thread-per-atom kernel's pack plan may use; batches whose largest trajectory exceeds
   it stay on the warp-per-atom kernel (no replacement in the reference). */
int32_t mdt_nn_radial_block(mdt_ctx *ctx, int32_t max_block);

/* Verlet skin (A) of the fast kernels' neighbour lists (default 1.0; 0 = build every
   step).  Lists are rebuilt when an atom of the bead moved more than half the skin
   since the last build; the per-step list is filtered from it with the same exact
   cutoff test, so results do not depend on the skin. */
int32_t mdt_nn_set_skin(mdt_ctx *ctx, double skin_ang);

/* Re-pack the thread-per-atom kernel's CTAs over the trajectories still running
   (status MDT_TRAJ_RUNNING): stopped trajectories no longer hold threads of a CTA, so a batch
   whose trajectories leave at different times keeps its CTAs full.  The plan is rebuilt over
   all trajectories after mdt_state_upload and after an mdt_refill that restarted any.
   npacks (may be NULL) receives the number of CTAs (packs) of the plan, 0 when the batch
   does not run on that kernel (nothing to do).  No replacement in the reference, which runs
   one trajectory at a time. */
int32_t mdt_nn_repack(mdt_ctx *ctx, int32_t *npacks);

/* Autotuner of the thread-per-atom kernel (no counterpart in the reference): times nsteps
   fused MD steps (mdt_md_steps with p and precision MDT_PREC_FP32, MDT_PREC_BF16 or
   MDT_PREC_BF16X3) of the current batch for every candidate launch shape -- the largest CTA
   of the pack plan (256, 384 or 512 atoms: waves and warps per SM) times the Verlet skin
   (0.3, 0.5, 0.75, 1 A) --
   each from the same saved state, keeps the fastest (as mdt_nn_radial_block and
   mdt_nn_set_skin would set it) and restores the state, so the batch continues as if the
   call had not happened.  Results do not depend on the choice.  block, skin_ang and
   ms_per_step (may be NULL) receive the choice and its time.  MDT_ERR_UNSUPPORTED when the
   batch does not run on that kernel. */
int32_t mdt_autotune(mdt_ctx *ctx, int32_t precision, int32_t nsteps, const mdt_prop_params *p, int32_t *block,
                     double *skin_ang, double *ms_per_step);

/* per trajectory: number of bead evaluations that fell back to EMT, and 1 if a
   neighbour list overflowed max_neighbors (either may be NULL) */
int32_t mdt_nn_stats(mdt_ctx *ctx, int32_t *fallbacks, int32_t *overflow);

/* Raw (unscaled) symmetry functions of every bead-atom, G[slot*maxsf + s] with slots in
   Fortran (nb, N) order per trajectory; computes energies as a side effect (like
   RuNNer's mode 1, which derives scaling.data from them). */
int32_t mdt_nn_descriptors(mdt_ctx *ctx, int32_t precision, double *G);

/* neighbour lists of the last network evaluation, bead 1 of every trajectory:
   counts[total atoms], words[total atoms * max_neighbors] packed as
   j | (n1+8)<<16 | (n2+8)<<20 | (n3+8)<<24 (0-based atom j, image n1..n3), in the order
   of RuNNer_src/neighbor_para_short.f90:117-163 */
int32_t mdt_nn_neighbors(mdt_ctx *ctx, int32_t *counts, int32_t *words);

/* ---- training of the network (learned EMT surrogate) -------------------------
 * No counterpart in the reference's MD path (its fit.f90 fits EMT/REBO parameters
 * with MKL).  Every trajectory of the current batch is one training configuration
 * (nbeads must be 1).  Loss per configuration:
 *   w_energy * ((E - E_ref)/N)^2 + w_force * sum |F - F_ref|^2 / (3N)   (eV, eV/A),
 * averaged over the configurations of a step; Adam on FP32 master weights.
 * Requires scale_symmetry_functions, no centering, no normalize_nodes. */
typedef struct mdt_train_opts {
    double w_energy, w_force;
    double lr, beta1, beta2, eps;
    int32_t precision;          /* MDT_PREC_FP32 for training, MDT_PREC_FP64 for gradient checks,
                                   MDT_PREC_BF16: the network's forward, backward, tangent and
                                   weight-gradient products as BF16 GEMMs on the tensor cores
                                   (FP32 accumulation and master weights; two hidden layers of
                                   <= 32 nodes, <= 48 descriptors); MDT_PREC_BF16X3: the same
                                   with split operands (hi*hi + hi*lo + lo*hi, about 16 bits),
                                   for networks whose energy error is below BF16 rounding */
} mdt_train_opts;

/* Labels: energy[T] (eV), forces (3, 1, N) per trajectory (eV/A).  Computes the raw
   symmetry functions and neighbour lists once and starts the optimiser from the
   installed network's weights. */
int32_t mdt_train_set_labels(mdt_ctx *ctx, const double *energy, const double *forces);
/* One optimiser step on configurations conf_ids[n] (0-based trajectory indices).
   stats (may be NULL): [mean ((E-E_ref)/N)^2 in eV^2, mean squared force error per
   component in (eV/A)^2, loss]. */
int32_t mdt_train_step(mdt_ctx *ctx, const mdt_train_opts *opts, const int32_t *conf_ids, int32_t n, double *stats);
/* Gradient of the mean loss over conf_ids with respect to the weights (nelem *
   maxweights doubles, calconenn order per element), without updating them. */
int32_t mdt_train_gradient(mdt_ctx *ctx, const mdt_train_opts *opts, const int32_t *conf_ids, int32_t n,
                           double *grad);
/* Install the current master weights as the network used by mdt_calc_force /
   mdt_md_steps; weights (may be NULL) receives them (nelem * maxweights doubles). */
int32_t mdt_train_commit(mdt_ctx *ctx, double *weights);

/* ---- batch geometry --------------------------------------------------------
 * Replaces the universe constructor new_atoms (src/universe_mod.f90:77-115) for T
 * trajectories at once.  natoms[T], nbeads[T]; idx: 1-based type per atom
 * (concatenated); mass: per atom in eV fs^2/A^2 (amu * 103.638239276);
 * is_fixed: (3, nb, N) per trajectory, 1 = frozen; simbox: 9 doubles per trajectory
 * (column-major (3,3), cell vectors as columns); algo/is_proj: per type.
 * Projectile atoms must precede lattice atoms, as md_init's merge_universes makes them
 * (src/md_init.f90:559-625). */
int32_t mdt_batch_define(mdt_ctx *ctx, int32_t ntraj, const int32_t *natoms, const int32_t *nbeads,
                         const int32_t *idx, const double *mass, const uint8_t *is_fixed,
                         const double *simbox, int32_t ntypes, const int32_t *algo, const uint8_t *is_proj);

/* Upload positions / velocities (Fortran order, see above); resets trajectory status. */
int32_t mdt_state_upload(mdt_ctx *ctx, const double *r, const double *v);
/* Download any subset (NULL skips).  dens is (nb, N) per trajectory: the EMT embedded
   density, or the friction coefficient after propagate_2 for LDFA atoms (the
   reference's shared `dens` array, pes_emt_mod.f90:45 / md_algo.f90:556-558). */
int32_t mdt_state_download(mdt_ctx *ctx, double *r, double *v, double *f, double *a, double *epot,
                           double *dens);

/* ---- hot path --------------------------------------------------------------
 * calc_force (src/force.f90:40-86): zero f/a/epot, free ring-polymer step when
 * nbeads > 1 (force.f90:54), EMT energies and forces, a = f/m for mobile atoms. */
int32_t mdt_calc_force(mdt_ctx *ctx, int32_t flag, int32_t precision, const mdt_prop_params *p);
/* propagate_1 / propagate_2 (src/md_algo.f90:37-106) */
int32_t mdt_propagate_1(mdt_ctx *ctx, const mdt_prop_params *p);
int32_t mdt_propagate_2(mdt_ctx *ctx, const mdt_prop_params *p);
/* nsteps of propagate_1 -> calc_force -> propagate_2 with the exit test
   (md_tian2.f90:78-92) in one fused launch. */
int32_t mdt_md_steps(mdt_ctx *ctx, int32_t nsteps, int32_t precision, const mdt_prop_params *p);

/* Deviates for rng_mode 1, each in Fortran order per trajectory: randy/zeta/andersen_v
   (3, nb, N) normal deviates, andersen_u (nb, N) uniforms.  NULL leaves one unset. */
int32_t mdt_set_random_arrays(mdt_ctx *ctx, const double *randy, const double *zeta, const double *andersen_v,
                              const double *andersen_u);

/* Per-trajectory step limit of the fused MD steps (the reference's nsteps): a trajectory
   that has run max_steps steps stops with status MDT_TRAJ_STEP_LIMIT (0 = no limit). */
int32_t mdt_set_step_limit(mdt_ctx *ctx, int32_t max_steps);

/* Refill (prepare_next_traj, src/md_init.f90:880-944, on the device): every trajectory that
   ended normally (status MDT_TRAJ_EXIT_UPPER, _EXIT_LOWER or _STEP_LIMIT) gets the state of the
   last mdt_state_upload back, and its projectile (atom 0) a new start the way apply_pip
   (md_init.f90:546-549) and set_proj_incidence (:829-876) place it: the bead centroid moves to
   a uniform position in the plane of the first two cell vectors at height z0 (every bead moves
   by target - centroid, so the ring polymer keeps its spread) and the bead velocities lose
   their mean and gain the incidence velocity for an energy uniform in [einc_min, einc_max] eV,
   a polar angle uniform in [polar_min, polar_max] degrees and the azimuth (degrees; < 0:
   uniform), drawn from a counter-based generator keyed by (seed, trajectory, generation).
   Trajectories with an error status (MDT_TRAJ_ERR_*) keep their state and status, so the
   caller sees them.  Status, step count and trajectory observables restart; generation[t]
   (may be NULL) counts the refills of each trajectory.  Forces are stale afterwards: call
   mdt_calc_force before the next mdt_md_steps, as after an upload.
   Differences from prepare_next_traj, which reads a new slab file and a new projectile file
   for every trajectory and draws einc from N(einc, sigma_einc): a trajectory slot restarts
   from its own uploaded slab every time (one slab microstate per slot; upload a new state to
   change it), and einc is uniform.  Lets a batch run a stream of trajectories on the GPU
   without uploading new states (the reference runs one trajectory at a time). */
typedef struct mdt_refill_params {
    double z0;
    double einc_min, einc_max;
    double polar_min, polar_max;
    double azimuth;
    uint64_t seed;
} mdt_refill_params;
int32_t mdt_refill(mdt_ctx *ctx, const mdt_refill_params *p, int32_t *generation, int32_t *nrefilled);
/* What the last mdt_refill drew for each trajectory: draws[5 t .. 5 t + 4] = the direct
   in-plane coordinates u, v of the new centroid, the incidence energy (eV), the polar and
   the azimuth angle (degrees); NaN for trajectories it did not restart.  Lets a host replay
   the start with md_init's apply_pip / set_proj_incidence (no reference counterpart). */
int32_t mdt_refill_draws(mdt_ctx *ctx, double *draws);

/* Trajectory observables of collect_trajectory_characteristics (src/trajectory_info.f90:
   47-75, 92-132, 243-250), tracked on the device by the fused MD steps (mdt_md_steps) after
   every step and reset by mdt_state_upload: per trajectory the turning points of the
   projectile centroid's z velocity, the closest approach (A) of the projectile (atom 0) to
   any other atom (minimum image of the centroids; the FP32 radial kernel takes the nearest
   entry of its neighbour list, within cutoff + skin) and the step at which it was first
   reached, and the lowest projectile centroid position r_min_p[3*t .. 3*t+2].  Any output
   may be NULL.  The reference's closest-approach time (the step times `step` once per
   later collect) follows from cl_appr_step on the host. */
int32_t mdt_traj_observables(mdt_ctx *ctx, int32_t *turn_pnts, double *cl_appr, int32_t *cl_appr_step,
                             double *r_min_p);

/* Bounce detection and adsorption of collect_trajectory_characteristics
   (src/trajectory_info.f90:80-263), tracked by the fused MD steps after every step and reset
   by mdt_state_upload / mdt_refill: bounces[t] counts the projectile's collisions (per
   nearest-atom segment the smallest of the r.v + to - sign changes and the crossings of r.v
   with r.F and with v.F, with the open segment closed as output_scatter closes it,
   output_mod.f90:660); interaction_time[t] (fs) the time with a non-zero projectile force;
   is_adsorbed[t] the adsorption flag (set when the closest approach of a step falls below
   the start limit, cleared above the end limit of mdt_set_adsorption).  Any output may be
   NULL; p supplies the step (fs). */
int32_t mdt_traj_bounces(mdt_ctx *ctx, int32_t *bounces, double *interaction_time, int32_t *is_adsorbed,
                         const mdt_prop_params *p);
/* The adsorption limits (A) of md_tian.inp's adsorption keyword (run_config.f90:644-650):
   adsorbed below `start`, free again above `end`; default: never adsorbed (the reference's
   default_real limits). */
int32_t mdt_set_adsorption(mdt_ctx *ctx, double start, double end);

/* per-trajectory status, steps and energies (output_mod.f90:658-697 fields) */
int32_t mdt_query(mdt_ctx *ctx, const mdt_prop_params *p, mdt_traj_summary *out);

/* device pointers of the SoA state (x,y,z arrays of r, v, f, a) for zero-copy callers;
   ptrs must hold 12 entries; *nslots receives the number of bead-atom slots. */
int32_t mdt_device_state(mdt_ctx *ctx, void **ptrs, int64_t *nslots);

/* ---- allocation-free EMT -------------------------------------------------------
 * No counterpart in the reference.  EMT energy, forces and embedded densities of ONE
 * configuration (one bead) for callers that must not allocate device memory -- a
 * program whose GPU memory is handed out by another runtime's pool, a loop that may
 * never enter the CUDA allocator, a caller without a library context.  Nothing is
 * allocated: the pair scratch lives in a 1.5 MiB file-scope device array that every
 * GPU loading the library keeps until process exit.  At most 256 atoms
 * (MDT_ERR_TOO_LARGE beyond).  All array arguments except simbox and the EMT
 * parameters are DEVICE pointers: idx (natoms, 1-based types), x/y/z positions (A),
 * outputs fx/fy/fz (eV/A, overwritten), energy (one double, eV, overwritten; NaN if a
 * type index is outside [1, ntypes]), dens (embedded density per atom, may be NULL).
 * simbox: host, 9 doubles column major.  EMT parameters and the pes table: host, as
 * for mdt_emt_set_params.  The call is asynchronous on `stream` (NULL = default
 * stream).  The first call on a device looks up the scratch array's address and must
 * come before any stream capture.  Calls share the scratch: calls that overlap on the
 * GPU race and must be serialised by the caller. */
int32_t mdt_emt_force_noalloc(int32_t natoms, const int32_t *idx, const double *x, const double *y,
                              const double *z, const double *simbox, int32_t ntypes, const double *eta2,
                              const double *n0, const double *e0, const double *lambda, const double *v0,
                              const double *kappa, const double *s0, const int32_t *pes, double *fx, double *fy,
                              double *fz, double *energy, double *dens, void *stream);

/* ---- measurement -------------------------------------------------------------
 * FMA throughput of the current device (FP64 or FP32 CUDA cores): the roofline
 * denominator of the EMT kernels, which are arithmetic-bound.  No reference
 * counterpart (the reference has no GPU code). */
int32_t mdt_peak_fma(int32_t precision, int32_t iters, double *flops_per_s);

/* The deviates the propagators draw, for statistical checks of the generator (the
 * reference's counterpart is its normal deviate, src/useful_things.f90:121-173, Box-Muller
 * in FP64 on the compiler's random_number).  out[i] = the deviate of (seed, traj, step,
 * slot i, stream) for i < n: kind 0 the N(0,1) deviate of the Langevin/PILE/Andersen noise
 * (Box-Muller in FP32 on 24-bit uniforms of a Philox4x32-10 block), kind 1 the uniform in
 * [0, 1) with 53 random bits; stream 1 Langevin, 2 PILE, 3 Andersen velocities, 4 Andersen
 * uniforms, 5 refill.  n <= 2^32; allocates and frees its own device buffer. */
int32_t mdt_rng_deviates(int32_t kind, uint64_t seed, int32_t traj, int32_t step, int32_t stream, int64_t n,
                         double *out);

/* The bounded wait of the tensor-core network (every mbarrier wait of a GEMM round gives up
 * after max_polls tries, 0 = the kernels' own limit, sets an error word that mdt_synchronize
 * reports, and the kernel returns instead of stalling), run alone on one CTA: with arrive = 0
 * nothing completes the barrier and timed_out must come back 1, with arrive = 1 a thread
 * arrives first and it must come back 0; ms (may be NULL) receives the kernel's time.
 * Lets a caller check on its own GPU that a lost MMA completion ends in an error status,
 * not a hang.  No reference counterpart (the reference has no GPU code). */
int32_t mdt_wait_check(int32_t max_polls, int32_t arrive, int32_t *timed_out, double *ms);

/* ---- work counters ---------------------------------------------------------- */
/* number of kernel launches this context issued since creation */
int64_t mdt_launch_count(const mdt_ctx *ctx);

#ifdef __cplusplus
}
#endif

#endif /* MDT_GPU_H */
