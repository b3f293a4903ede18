/*
 * mpcmd — GB300-native hybrid MD / reactive multiparticle-collision engine.
 *
 * C ABI of the drop-in boundary.  The reference program (rober468/main
 * collective_code/main_pattern.f95 and selkov_code/Main_SelkovDimer.f90) calls
 * Fortran module subroutines on host arrays; this library keeps the whole
 * state resident on one GPU and exposes one entry point per reference module
 * call.  A Fortran driver binds these with iso_c_binding (see
 * fortran/mpcmd_shim.f90); Python binds them with ctypes (main_gb300).
 *
 * Conventions: particle and cell indices are 0-based; sphere s = 2k + i for
 * dimer k with i = 0 the catalytic (C) and i = 1 the non-catalytic (N) sphere;
 * positions are in units of the MPC cell (a0 = 1).  Every function returns an
 * mpcmd_status; no function aborts the process.  A context is not thread-safe
 * and owns one CUDA stream on the current device.
 */
#ifndef MPCMD_H
#define MPCMD_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mpcmd_status {
  MPCMD_OK = 0,
  MPCMD_ERR_CONFIG = 1,            /* invalid or unsupported configuration          */
  MPCMD_ERR_ALLOC = 2,             /* device or host allocation failed              */
  MPCMD_ERR_CELL_OVERFLOW = 3,     /* a cell holds more than cell_capacity of a species */
  MPCMD_ERR_NEIGHBOUR_OVERFLOW = 4,/* shell buffers or per-particle sphere slots full */
  MPCMD_ERR_RATTLE = 5,            /* bond constraint hit rattle_max_iter           */
  MPCMD_ERR_INIT = 6,              /* initial placement did not converge            */
  MPCMD_ERR_STATE = 7,             /* call out of order (e.g. step before prepare)  */
  MPCMD_ERR_CUDA = 8,              /* a CUDA runtime call failed                    */
  MPCMD_ERR_IO = 9,                /* checkpoint file could not be written or read  */
  MPCMD_ERR_CHECKPOINT = 10        /* checkpoint file is corrupt or does not match  */
} mpcmd_status;

enum { MPCMD_GEOM_WALLS = 0, MPCMD_GEOM_PERIODIC = 1 };
enum { MPCMD_KIN_NONE = 0, MPCMD_KIN_SIMPLE = 1, MPCMD_KIN_SELKOV = 2 };
enum { MPCMD_EXCL_PARTICLE = 0, MPCMD_EXCL_CELLS = 1 };
/* Catalysis on the C sphere: DETERMINISTIC, A -> B at the first force
 * evaluation inside the C cutoff (forces_mod.f95:79-81); PROBABILISTIC, the
 * draws of ForcesMD_SelkovDimer.f90:143-198; ON_EXIT, A -> B (probability 1)
 * when a particle inside a C cutoff at one force evaluation is outside every
 * C cutoff at the next (the rule of the plain single-dimer workload; not in
 * the reference's code; owner tags require DETERMINISTIC).  A restart starts
 * with no particle recorded inside: its force evaluation records them. */
enum { MPCMD_CAT_DETERMINISTIC = 0, MPCMD_CAT_PROBABILISTIC = 1, MPCMD_CAT_ON_EXIT = 2 };
enum { MPCMD_PREC_FP32 = 32, MPCMD_PREC_FP64 = 64 };
/* rotational_code variants: MOTOR is the free dimer of collective_code and
 * selkov_code; ROTOR is the anchored dimer of rotational_code/2d_array and
 * linear_periodic_ci (see `variant` below).  Layouts of mpcmd_initial: random
 * placement (initial_mod.f95:78-119), a rows x cols grid
 * (rotational_code/2d_array/initial_mod.f95:68-90) or a line along x
 * (rotational_code/linear_periodic_ci/initial_mod.f95:72-88). */
enum { MPCMD_VARIANT_MOTOR = 0, MPCMD_VARIANT_ROTOR = 1 };
enum { MPCMD_LAYOUT_RANDOM = 0, MPCMD_LAYOUT_GRID = 1, MPCMD_LAYOUT_LINE = 2 };

/* Run configuration.  The first block (through k[6]) carries the reference
 * input decks (collective_code/input.txt read at main_pattern.f95:19-64,
 * selkov_code/Input_SelkovDimer read at Main_SelkovDimer.f90:7-45) after the
 * derivations of main_pattern.f95:66-127. */
typedef struct mpcmd_config {
  int32_t lx, ly, lz;        /* box edges in cells                                   */
  int32_t geometry;          /* MPCMD_GEOM_*: z walls (collective) or periodic        */
  int32_t n_dimers;          /* numdims                                             */
  int32_t kinetics;          /* MPCMD_KIN_*: reaction_simple or Selkov RKMPC         */
  int32_t exclusion;         /* MPCMD_EXCL_*: distribute_mod bulk rule or Affected_Cell */
  int32_t catalysis;         /* MPCMD_CAT_*: forces_mod.f95:79-92, ForcesMD:302-376 or on exit */
  int32_t rotation_sense;    /* +1 mpc_rotation_mod Rodrigues, -1 RMPC projection     */
  int32_t mpc_every;         /* MPCtstep                                             */
  int32_t sort_every;        /* sort_step (0 = never)                                */
  int32_t react_box_type;    /* reactive floor pattern 1..7                          */
  int32_t react_dir;         /* 0: A->B on the floor, 1: B->A                        */
  int32_t cell_capacity;     /* MaxA (per-cell per-species capacity, <= 255)         */
  int32_t max_neighbour;     /* max_neighbour (per-sphere list capacity)             */
  int32_t rattle_max_iter;   /* Con1Max / Con2Max                                    */
  int32_t init_plane;        /* 1: mpcmd_initial places dimers in the z mid-plane    */
  int32_t pad0;
  int64_t n_solvent;         /* NT                                                   */
  uint64_t seed;             /* key of the counter-based random streams              */
  int64_t init_count[4];     /* Na0, Nb0, Ns0 (species codes 0..3) for mpcmd_initial */
  double mass[4];            /* Ma, Mb, Ms (per species code)                        */
  double eps_c[4];           /* EaC, EbC, EsC                                        */
  double eps_n[4];           /* EaN, EbN, EsN                                        */
  double rc, rn, dcn;        /* Rc, Rn, Dcn                                          */
  double mc, mn;             /* Mc, Mn                                               */
  double rw, ew;             /* Rw, Ew                                               */
  double rm_delta, em;       /* Rm_delta, Em                                         */
  double rp_ab, rp_ba;       /* RPab, RPba                                           */
  double kT, skin, rot_angle, md_dt, mpc_dt;  /* T, skinrad, rotang, MDt, MPCt       */
  double k[6];               /* k1 (simple) or k1..k6 (Selkov)                       */
  /* GB300 engine options (not in the reference decks). */
  int32_t precision;         /* MPCMD_PREC_FP32 (default) or MPCMD_PREC_FP64         */
  int32_t shell_capacity;    /* 0 = sized from the sphere shells                     */
  /* rotational_code variants (rotational_code/2d_array/main_rotation.f95:17-69). */
  int32_t variant;           /* MPCMD_VARIANT_ROTOR: every dimer's midpoint is held at
                                its anchor (RATTLE of 2d_array/evolve_mod.f95:283-391,
                                596-650), a harmonic z tether on each sphere
                                (forces_mod.f95:177-201) replaces the 9-3 wall, and
                                there is no motor-motor LJ                          */
  int32_t layout;            /* MPCMD_LAYOUT_*: dimer placement of mpcmd_initial     */
  int32_t layout_rows, layout_cols;  /* numrows, numcols of the grid layout          */
  int32_t owner_tags;        /* 1: type_B of linear_periodic_no_ci (forces_mod.f95:79-121):
                                the C sphere of motor k makes every particle in its
                                cutoff a B of motor k, and a B acts as A on the
                                spheres of every other motor (deterministic catalysis,
                                simple kinetics, no reactive floor)                  */
  int32_t reserved;
  double tether_k, tether_z; /* k_harm, zdimeq (= Rc + gap)                          */
  double layout_sep;         /* sep: gap between neighbouring motors of a layout     */
} mpcmd_config;

typedef struct mpcmd_obs {
  double momentum[3];        /* total (solvent + spheres), FP64 reduction            */
  double solvent_momentum[3];
  double kinetic_solvent, kinetic_dimer, potential;
  int64_t species_count[4];
  int64_t n_inside, n_pairs;
  int32_t time_count, time_penetrate;
  int64_t cstep;
} mpcmd_obs;

typedef struct mpcmd_ctx mpcmd_ctx;

/* Lifetime ------------------------------------------------------------ */
int mpcmd_create(const mpcmd_config* cfg, mpcmd_ctx** out);
int mpcmd_destroy(mpcmd_ctx* ctx);
const char* mpcmd_error_string(int status);
int mpcmd_device_bytes(const mpcmd_ctx* ctx, int64_t* bytes);

/* State exchange (host SoA in the reference's FP64 layout) ------------- */
/* global_mod.f95:95-111 arrays Xsol..VZsol, flag; Xdim..FZdim as [2*nd][3]. */
int mpcmd_upload_state(mpcmd_ctx* ctx, const double* x, const double* y, const double* z,
                       const double* vx, const double* vy, const double* vz,
                       const int32_t* flag, const double* dpos, const double* dvel,
                       const double* dforce);
int mpcmd_download_state(mpcmd_ctx* ctx, double* x, double* y, double* z,
                         double* vx, double* vy, double* vz, int32_t* flag,
                         double* dpos, double* dvel, double* dforce);
/* Cell visiting order of the sort (hilbert.txt, sort_hilbert_mod.f95:57-62):
 * order[k] = 0-based row-major id of the k-th cell.  Without it the engine
 * uses its own Hilbert order. */
int mpcmd_set_cell_order(mpcmd_ctx* ctx, const int32_t* order, int64_t n);
/* Anchors of the rotor variant, motorCM [3*n_dimers]
 * (rotational_code/2d_array/initial_mod.f95:86-88, restart_mod.f95 reads them
 * back from motor_positions.dat).  mpcmd_initial and mpcmd_upload_state set
 * them to the midpoints 0.5 (X_C + X_N) of the dimers they place or receive;
 * mpcmd_restore sets the checkpointed ones. */
int mpcmd_set_anchors(mpcmd_ctx* ctx, const double* anchors);
int mpcmd_get_anchors(mpcmd_ctx* ctx, double* anchors);
/* Owner tags type_B [n_solvent]: the 1-based motor number of the C sphere
 * that made a B particle, 0 for none (linear_periodic_no_ci/global_mod.f95:72).
 * mpcmd_initial and mpcmd_upload_state clear them; the tags follow the
 * particles through the sort (sort_hilbert_mod.f95:75) and are cleared by the
 * B -> A reaction (reaction_simple_mod.f95:55).  MPCMD_ERR_CONFIG without
 * owner_tags. */
int mpcmd_set_owner_tags(mpcmd_ctx* ctx, const int32_t* type_b);
int mpcmd_get_owner_tags(mpcmd_ctx* ctx, int32_t* type_b);
int mpcmd_set_step(mpcmd_ctx* ctx, int64_t cstep, int32_t time_count);
/* Collision angle, interval and rate constants k[6] (may be NULL: rates
 * unchanged), as a driver passes rotang to mpc_rotation
 * (mpc_rotation_mod.f95:6) and MPCt, k1 to reaction_simple
 * (reaction_mod.f95:8); they apply from the next collision. */
int mpcmd_set_collision(mpcmd_ctx* ctx, double rot_angle, double mpc_dt, const double* k);
/* Order-only re-sort every `every` MD steps (a multiple of mpc_every; 0 =
 * never; default 10 * mpc_every).  At the start of such a collision step the
 * particles are regrouped in memory by the cell order of sort_hilbert_mod
 * (the reference's own sort stays at sort_every, sort_hilbert_mod.f95:6-98).
 * Nothing observable changes: every particle keeps its main index, which
 * orders the species lists (distribute_mod.f95:95-182), keys the catalysis
 * draws and indexes every per-particle array this interface reads or writes.
 * Returns MPCMD_ERR_CONFIG for a negative value or one that is not a multiple
 * of mpc_every. */
int mpcmd_set_resort(mpcmd_ctx* ctx, int64_t every);
/* The reactive floor as the driver's react_box array [lx * ly], nonzero =
 * reactive patch (reactive_grid_mod.f95:8-99 fills it; evolve reads it). */
int mpcmd_set_reactive_grid(mpcmd_ctx* ctx, const int32_t* table);

/* Reference call surface ----------------------------------------------- */
int mpcmd_initial(mpcmd_ctx* ctx);        /* initial_mod.f95:6-355                 */
int mpcmd_prepare(mpcmd_ctx* ctx);        /* main_pattern.f95:168-187              */
/* restart_mod.f95:415-528: mpcmd_prepare, then the forces of the state (pair
 * forces for the first half kick, catalysis, sphere totals) without a kick.
 * mpcmd_prepare after mpcmd_restore does the same. */
int mpcmd_prepare_restart(mpcmd_ctx* ctx);
int mpcmd_step(mpcmd_ctx* ctx);           /* main_pattern.f95:203-225, one step    */
int mpcmd_evolve(mpcmd_ctx* ctx);         /* evolve_mod.f95:6-732, one MD step only */
int mpcmd_run(mpcmd_ctx* ctx, int64_t nsteps);  /* nsteps main-loop iterations     */
int mpcmd_sort(mpcmd_ctx* ctx);           /* sort_hilbert_mod.f95:6-98             */
int mpcmd_rebuild_lists(mpcmd_ctx* ctx);  /* neighbour_list_mod.f95:6-184          */
int mpcmd_distribute(mpcmd_ctx* ctx);     /* distribute_mod.f95 / Affected_Cell.f90 */
int mpcmd_mpc_rotation(mpcmd_ctx* ctx);   /* mpc_rotation_mod.f95 / RMPC:15-120     */
int mpcmd_reaction(mpcmd_ctx* ctx);       /* reaction_mod.f95:8-66 / RMPC:127-324   */
int mpcmd_observables(mpcmd_ctx* ctx, mpcmd_obs* out);  /* output_mod.f95:681-806   */
int mpcmd_checkpoint(mpcmd_ctx* ctx, const char* path); /* restart_mod.f95 state    */
int mpcmd_restore(mpcmd_ctx* ctx, const char* path);

/* Concentration fields (output_mod.f95:482-575): species A (code 0) and B
 * (code 1) counted in slabs of half thickness `half_width` (the reference
 * passes cutoffC) around x_slab / y_slab / z_slab, on bins of x_width,
 * y_width, z_width.  A particle at coordinate u is in bin ceiling(u / width)
 * (1-based; a coordinate of exactly 0 goes to bin 1, where the reference
 * would index 0), and in a slab when |u - slab| <= half_width.  Counts are
 * divided by the bin volumes of the reference.  Positions are the host view
 * of mpcmd_download_state (outside particles at the last rebuild).  Outputs
 * (any may be NULL), nx = int(lx / x_width), ny, nz likewise, 2D arrays with
 * their first index fastest (Fortran order):
 *   totals[4]  TotA, TotB, ConcA = TotA / volume, ConcB
 *   c1d_a/b    [nx]      z slab, binned along x
 *   xy_a/b     [nx*ny]   z slab
 *   xz_a/b     [nx*nz]   y slab
 *   yz_a/b     [ny*nz]   x slab */
typedef struct mpcmd_conc_params {
  double x_slab, y_slab, z_slab;
  double half_width;
  double x_width, y_width, z_width;
} mpcmd_conc_params;
int mpcmd_concentration(mpcmd_ctx* ctx, const mpcmd_conc_params* p, double* totals,
                        double* c1d_a, double* c1d_b, double* xy_a, double* xy_b,
                        double* xz_a, double* xz_b, double* yz_a, double* yz_b);
/* Dimer axes: d = X_C - X_N with the minimum image on the periodic axes,
 * nucvec[3k..3k+2] = d / Dcn when normalize == 0 (output_mod.f95:826-846) or
 * d / |d| when normalize == 1 (Output_SelkovDimer.f90:146-166); vdot[k] (may
 * be NULL) = centre-of-mass velocity . unit axis, the propulsion speed of
 * Output_SelkovDimer.f90:168-172. */
int mpcmd_dimer_axes(mpcmd_ctx* ctx, int normalize, double* nucvec, double* vdot);

/* Inspection (parity tests) -------------------------------------------- */
int mpcmd_get_new_cell(mpcmd_ctx* ctx, int64_t* newcell);           /* NewCellN     */
int mpcmd_get_cell_rotation(mpcmd_ctx* ctx, double* cm, double* axis, int32_t* count);
int mpcmd_get_distribute(mpcmd_ctx* ctx, int32_t* counts, int64_t* first);
int mpcmd_get_affected(mpcmd_ctx* ctx, int32_t* affected);
int mpcmd_get_shift(mpcmd_ctx* ctx, double* shift);
/* Pairs (particle, sphere) of the shell buffer entries; between collision
 * steps, inside-list members in free flight (no LJ cutoff reachable before
 * the next collision rebuild) are kept outside the buffer and listed by
 * mpcmd_get_inside only. */
int mpcmd_get_pairs(mpcmd_ctx* ctx, int64_t* n_pairs, int64_t* particle, int32_t* sphere);
/* The inside list (neighbour_list_mod.f95 inout_particle_list) of the last rebuild. */
int mpcmd_get_inside(mpcmd_ctx* ctx, int64_t* n_inside, int64_t* idx);
/* Up to n of: shell entries, device status bits, time_penetrate, RATTLE
 * iterations, cstep, time_count, pending abort step, last rebuild step,
 * checked-build failure code and value, watch-list entries, and since the last
 * mpcmd_profile(ctx, 1): shell entries over all force launches, particles
 * visited over all rebuild launches, shell entries written by the rebuilds;
 * then the order-only re-sorts run since create. */
int mpcmd_get_counters(mpcmd_ctx* ctx, int64_t* counters, int32_t n);
int mpcmd_reactive_grid_table(mpcmd_ctx* ctx, int32_t* table);
int mpcmd_cell_order(mpcmd_ctx* ctx, int32_t* order);
int64_t mpcmd_kernel_launches(mpcmd_ctx* ctx);

/* Measurement ---------------------------------------------------------- */
/* Select the CUDA device of the contexts created afterwards by this thread. */
int mpcmd_set_device(int device);
/* Record event `slot` (0..7) on the context stream; elapsed time between two
 * recorded slots in milliseconds (waits for the later one). */
int mpcmd_event_record(mpcmd_ctx* ctx, int slot);
int mpcmd_event_elapsed(mpcmd_ctx* ctx, int a, int b, double* ms);
int mpcmd_synchronize(mpcmd_ctx* ctx);
/* Per-launch CUDA-event timing by kernel kind: 0 rebuild, 1 force, 2 dimer,
 * 3 cells, 4 rotate_main, 5 shell_advance, 6 bins, 7 finalize, 8 sort,
 * 9 affected.  Enabling clears the totals. */
int mpcmd_profile(mpcmd_ctx* ctx, int enable);
int mpcmd_profile_read(mpcmd_ctx* ctx, double* ms, int64_t* count, int n);

/* Allocation-free collision ------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot call cudaMalloc:
 * a host whose memory manager owns all device memory (a pool sized at
 * start-up or a framework allocator) and may not be bypassed, or a stepping
 * loop that cannot pay cudaMalloc/cudaFree's device synchronisation.  It
 * performs the FP64 collision stage of mpcmd_mpc_rotation (grid shift drawn
 * for `step`, per shifted cell centre of mass and random axis, rotation by
 * rot_angle) on caller-owned device arrays: x, y, z absolute positions in
 * cell units (inputs) and vx, vy, vz velocities (rotated in place), n
 * particles, box lx x ly x lz cells, geometry MPCMD_GEOM_*, rotation_sense
 * +1 (Rodrigues form) or -1 (projection form), contract seed.  Launches on
 * `stream` (a cudaStream_t; NULL = legacy default stream) and does not wait.
 * Allocates nothing: its only scratch is a static device array of
 * MPCMD_STATIC_MAX_CELLS x 4 doubles (16 MiB) that every GPU loading this
 * library holds until exit; boxes with more shifted cells (lx*ly*lz, or
 * lx*ly*(lz+1) with walls) return MPCMD_ERR_CONFIG.  The first call on a
 * device resolves the array's address (cudaGetSymbolAddress) and must come
 * before any stream capture; every uncaptured call resolves it again, so after
 * cudaDeviceReset make the next call outside a capture.  All calls on a device
 * share the array (each clears what it uses): calls that overlap on the GPU
 * race and must be serialised by the caller.  A CUDA error already pending on
 * the calling thread makes the call return MPCMD_ERR_CUDA without launching;
 * on MPCMD_ERR_CUDA the CUDA error is left for cudaGetLastError. */
#define MPCMD_STATIC_MAX_CELLS 524288
int mpcmd_collide_static(const double* x, const double* y, const double* z,
                         double* vx, double* vy, double* vz, int64_t n,
                         int32_t lx, int32_t ly, int32_t lz, int32_t geometry,
                         double rot_angle, int32_t rotation_sense, uint64_t seed,
                         int64_t step, void* stream);

/* Batched ensemble ------------------------------------------------------ */
/* Many independent single-dimer replicas of the plain periodic run
 * (collective_code physics with a periodic box: main_pattern.f95:203-225 per
 * replica, deterministic catalysis forces_mod.f95:79-81, reaction_simple
 * reaction_mod.f95:8-66, Rodrigues collision mpc_rotation_mod.f95:102-228),
 * each with its own box, density, sphere sizes, bond, interaction, rate and
 * seed, advanced together on one GPU.  The reference runs such replicas as
 * separate jobs of a job array
 * (rotational_code/linear_periodic_langevin/setup/5_make_subjobs.sh).  Every
 * replica follows the same step sequence as an mpcmd context of the same
 * configuration (geometry periodic, one dimer, kinetics simple, exclusion
 * particle, catalysis deterministic, rotation_sense +1) and the same contract
 * random streams, so a replica equals its own single-context run up to
 * rounding.  All replicas share md_dt, mpc_dt, rot_angle, skin, sort_every and
 * cell_capacity and advance in lockstep; each decides its own list rebuilds on
 * the device.  One launch per stage covers every replica; mpcmd_ens_run
 * replays each collision period as one CUDA graph. */
typedef struct mpcmd_replica {
  int32_t lx, ly, lz;        /* box edges in cells (4..1024)                        */
  int32_t reserved;
  int64_t n_solvent;         /* solvent particles (all species A at mpcmd_ens_initial) */
  uint64_t seed;             /* contract-stream key of this replica                 */
  double mass[4];            /* solvent mass per species code                       */
  double eps_c[4], eps_n[4]; /* LJ strengths of the C and N spheres per species      */
  double rc, rn, dcn;        /* sphere radii (sigma_C, sigma_N) and bond length      */
  double mc, mn;             /* sphere masses (0: density-matched, main_pattern.f95:118-119) */
  double kT;                 /* temperature of the initial velocities               */
  double k1;                 /* bulk B -> A rate (reaction_mod.f95:41-62)            */
} mpcmd_replica;

typedef struct mpcmd_ensemble_config {
  int32_t n_replicas;
  int32_t precision;         /* MPCMD_PREC_FP32 or MPCMD_PREC_FP64                   */
  int32_t sort_every;        /* sort_step in MD steps (0 = never)                    */
  int32_t cell_capacity;     /* per-cell per-species capacity (<= 255)               */
  int32_t rattle_max_iter;
  int32_t particle_tile;     /* particles per work tile (0 = from the autotuner cache or 2048) */
  int32_t block;             /* threads per block of the particle kernels (0 = 256)  */
  int32_t shell_block;       /* shell entries per tile = threads per block (0 = 256) */
  double md_dt, mpc_dt, rot_angle, skin;
} mpcmd_ensemble_config;

typedef struct mpcmd_ens mpcmd_ens;

int mpcmd_ens_create(const mpcmd_ensemble_config* cfg, const mpcmd_replica* replicas, mpcmd_ens** out);
int mpcmd_ens_destroy(mpcmd_ens* ens);
int mpcmd_ens_device_bytes(const mpcmd_ens* ens, int64_t* bytes);
/* initial_mod.f95:6-355 for every replica (the draws of mpcmd_initial). */
int mpcmd_ens_initial(mpcmd_ens* ens);
/* State of replica r in the reference layout (as mpcmd_upload_state /
 * mpcmd_download_state); dpos/dvel/dforce are [2][3]. */
int mpcmd_ens_upload(mpcmd_ens* ens, int32_t r, const double* x, const double* y, const double* z,
                     const double* vx, const double* vy, const double* vz, const int32_t* flag,
                     const double* dpos, const double* dvel, const double* dforce);
int mpcmd_ens_download(mpcmd_ens* ens, int32_t r, double* x, double* y, double* z, double* vx,
                       double* vy, double* vz, int32_t* flag, double* dpos, double* dvel,
                       double* dforce);
/* main_pattern.f95:168-187 for every replica: sort (at step 0), lists, time_penetrate. */
int mpcmd_ens_prepare(mpcmd_ens* ens);
/* nsteps main-loop iterations of every replica; whole collision periods
 * starting on a period boundary run as graph replays. */
int mpcmd_ens_run(mpcmd_ens* ens, int64_t nsteps);
/* Per replica: out[r] as mpcmd_observables. */
int mpcmd_ens_observables(mpcmd_ens* ens, mpcmd_obs* out);
/* Propulsion speed (Output_SelkovDimer.f90:168-172: centre-of-mass velocity
 * along the unit axis C - N) sampled at every collision step since the last
 * reset: mean[r], and the unit axes of the samples, axes[r][k][3] for
 * k < min(count, history) (history as given to mpcmd_ens_reset_samples). */
int mpcmd_ens_reset_samples(mpcmd_ens* ens, int32_t history);
int mpcmd_ens_samples(mpcmd_ens* ens, double* mean_speed, int64_t* count, float* axes);
/* Axisymmetric B concentration around each dimer (the steady field the
 * output_mod.f95:486-603 slabs sample, in the dimer frame): B particles
 * counted on nz x nr bins of the axial coordinate z in [-zmax, zmax) and the
 * radius r in [0, rmax) about the dimer midpoint and axis; accumulated at
 * each call, read as counts[r][nz * nr] (z fastest... see ensemble.py) with
 * the number of accumulated samples. */
int mpcmd_ens_field_accumulate(mpcmd_ens* ens, int32_t nz, int32_t nr, double zmax, double rmax);
int mpcmd_ens_field_read(mpcmd_ens* ens, uint32_t* counts, int64_t* samples);
/* Work schedule: particle tile, block size of the particle kernels, shell
 * tile (= block) of the shell kernels.  mpcmd_ens_autotune times candidate
 * schedules on a snapshot of the state (restored afterwards) and keeps the
 * fastest; with a cache path it first looks up the shape class of the
 * ensemble there and records what it measured. */
int mpcmd_ens_set_schedule(mpcmd_ens* ens, int32_t particle_tile, int32_t block, int32_t shell_block);
int mpcmd_ens_get_schedule(mpcmd_ens* ens, int32_t* sched /* [3] */);
int mpcmd_ens_autotune(mpcmd_ens* ens, const char* cache_path, int32_t periods);
/* Up to n of: kernel launches, graph replays, device status bits, RATTLE
 * iterations, rebuilds over all replicas, cstep. */
int mpcmd_ens_counters(mpcmd_ens* ens, int64_t* counters, int32_t n);
int mpcmd_ens_event_record(mpcmd_ens* ens, int slot);
int mpcmd_ens_event_elapsed(mpcmd_ens* ens, int a, int b, double* ms);
int mpcmd_ens_synchronize(mpcmd_ens* ens);

/* Learned surrogate --------------------------------------------------- */
/* A multilayer perceptron (n_in inputs -> n_layers hidden layers of width
 * n_hidden with SiLU -> n_out outputs) trained and evaluated by this
 * library's own kernels: every contraction runs on the fifth-generation
 * tensor cores (tcgen05.mma, BF16 operands staged by TMA, FP32 accumulators
 * in tensor memory); the weights are BF16 in the GEMMs with an FP32 master
 * copy for Adam.  No counterpart in the reference: it maps replica
 * parameters to the observables the reference's output routines define
 * (propulsion speed Output_SelkovDimer.f90:168-172, orientation correlation
 * 1D_Orientation_Correlation.py:40-53, concentration fields
 * output_mod.f95:486-603).  x, t, w and y are device pointers (FP32,
 * row-major); the calls return after their kernels have finished. */
typedef struct mpcmd_mlp_config {
  int32_t n_in;              /* 1..64                                               */
  int32_t n_hidden;          /* multiple of 64, 64..256                             */
  int32_t n_layers;          /* hidden layers, 1..16                                */
  int32_t n_out;
  int32_t batch;             /* training batch, multiple of 128                     */
  int32_t max_rows;          /* largest mpcmd_mlp_forward batch                     */
  uint64_t seed;             /* Glorot-uniform initial weights                      */
  double lr, beta1, beta2, eps;   /* Adam                                          */
} mpcmd_mlp_config;

typedef struct mpcmd_mlp mpcmd_mlp;

int mpcmd_mlp_create(const mpcmd_mlp_config* cfg, mpcmd_mlp** out);
int mpcmd_mlp_destroy(mpcmd_mlp* m);
/* Parameters in FP32, per layer W [n_out_l x n_in_l] row-major then b [n_out_l]. */
int mpcmd_mlp_param_count(const mpcmd_mlp* m, int64_t* n);
int mpcmd_mlp_get_params(mpcmd_mlp* m, float* host);
int mpcmd_mlp_set_params(mpcmd_mlp* m, const float* host);
/* y [rows, n_out] = network(x [rows, n_in]), rows <= max(batch, max_rows). */
int mpcmd_mlp_forward(mpcmd_mlp* m, const float* x, int64_t rows, float* y);
/* Loss sum_j w_j (y_j - t_j)^2 averaged over the batch (x [batch, n_in],
 * t [batch, n_out], w [n_out]) and its gradients, in the parameter layout
 * (host array, may be NULL); no update. */
int mpcmd_mlp_gradients(mpcmd_mlp* m, const float* x, const float* t, const float* w, float* grads,
                        double* loss);
/* One Adam step on a batch; loss (may be NULL) before the step. */
int mpcmd_mlp_train_step(mpcmd_mlp* m, const float* x, const float* t, const float* w, double* loss);
int mpcmd_mlp_synchronize(mpcmd_mlp* m);

/* Contract random numbers (same streams as the engine), for checkers. */
double mpcmd_contract_u01(uint64_t seed, uint32_t tag, uint32_t index, uint32_t extra,
                          uint32_t step, int which);

#ifdef __cplusplus
}
#endif
#endif
