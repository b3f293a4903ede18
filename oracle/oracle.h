/*
 * CPU oracle for the hybrid MD / reactive-MPC time step (test infrastructure).
 *
 * This is a plain-C FP64 restatement of the rober468/main Fortran modules, used
 * ONLY as the parity checker by tests/, by __graft_entry__.smoke() and as the
 * timed CPU baseline in bench.py.  It is never linked into the product library.
 *
 * Parity status: pinned by (a) MT19937 known answers (numpy's independent
 * MT19937 implementation), (b) Philox4x32-10 known-answer vectors of the
 * published algorithm, (c) the reference's own hilbert.txt cell order fixture,
 * (d) analytic known answers taken from the reference code (SRD diffusion
 * coefficient, collision invariants, RKMPC firing probability, RATTLE
 * tolerances).  No output of the reference program itself exists or can be
 * produced here (no Fortran compiler), so trajectory-level parity against the
 * Fortran binary is unpinned.
 *
 * Conventions: particle and cell indices are 0-based.  Sphere s = 2*k + i for
 * dimer k, i = 0 (catalytic C) or 1 (non-catalytic N).
 */
#ifndef MPCMD_ORACLE_H
#define MPCMD_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_GEOM_WALLS = 0, ORC_GEOM_PERIODIC = 1 };
enum { ORC_KIN_NONE = 0, ORC_KIN_SIMPLE = 1, ORC_KIN_SELKOV = 2 };
enum { ORC_EXCL_PARTICLE = 0, ORC_EXCL_CELLS = 1 };
/* ON_EXIT: A -> B when a particle inside a C cutoff at one force evaluation
 * is outside every C cutoff at the next (the plain single-dimer workload's
 * rule; the reference converts on entry, forces_mod.f95:79-81). */
enum { ORC_CAT_DETERMINISTIC = 0, ORC_CAT_PROBABILISTIC = 1, ORC_CAT_ON_EXIT = 2 };
enum { ORC_RNG_CONTRACT = 0, ORC_RNG_MT = 1 };
/* Pair search of orc_rebuild_lists: every particle against every sphere
 * (neighbour_list_mod.f95, the default), or through cell bins (the same
 * lists in the same order; a faster CPU baseline for comparison). */
enum { ORC_LISTS_ALL_PAIRS = 0, ORC_LISTS_CELLS = 1 };
/* rotational_code variants: ROTOR anchors every dimer's midpoint
 * (rotational_code/2d_array); dimer layouts of the initial placement. */
enum { ORC_VARIANT_MOTOR = 0, ORC_VARIANT_ROTOR = 1 };
enum { ORC_LAYOUT_RANDOM = 0, ORC_LAYOUT_GRID = 1, ORC_LAYOUT_LINE = 2 };

/* Random-stream tags of the counter-based contract RNG (shared with the GPU). */
enum {
  ORC_TAG_SHIFT = 1, ORC_TAG_AXIS = 2, ORC_TAG_RXN = 3, ORC_TAG_CAT = 4,
  ORC_TAG_INIT_DIMER = 5, ORC_TAG_INIT_POS = 6, ORC_TAG_INIT_VEL = 7
};

/* Error codes (same numbering as the product C ABI). */
enum {
  ORC_OK = 0, ORC_ERR_CONFIG = 1, ORC_ERR_ALLOC = 2, ORC_ERR_CELL_OVERFLOW = 3,
  ORC_ERR_NEIGHBOUR_OVERFLOW = 4, ORC_ERR_RATTLE = 5, ORC_ERR_INIT = 6,
  ORC_ERR_STATE = 7
};

/* Run parameters.  Field order and types are identical to mpcmd_config in
 * include/mpcmd.h so one ctypes mirror fills both. */
typedef struct orc_params {
  int32_t lx, ly, lz;        /* box edges in MPC cells (cell size a0 = 1)          */
  int32_t geometry;          /* ORC_GEOM_*                                          */
  int32_t n_dimers;
  int32_t kinetics;          /* ORC_KIN_*                                           */
  int32_t exclusion;         /* ORC_EXCL_*                                          */
  int32_t catalysis;         /* ORC_CAT_*                                           */
  int32_t rotation_sense;    /* +1 Rodrigues matrix form, -1 projection/cross form  */
  int32_t mpc_every;         /* MPCtstep: MD steps per collision                    */
  int32_t sort_every;        /* sort_step: MD steps between cell-order sorts (0=never) */
  int32_t react_box_type;    /* reactive floor pattern 1..7 (walls geometry only)    */
  int32_t react_dir;         /* 0: A->B on the floor, 1: B->A                       */
  int32_t cell_capacity;     /* per-cell per-species list capacity (MaxA)           */
  int32_t max_neighbour;     /* per-sphere neighbour list capacity                  */
  int32_t rattle_max_iter;   /* iteration cap of both RATTLE loops                  */
  int32_t init_plane;        /* 1: dimers placed in the z mid-plane, bond in xy     */
  int32_t pad0;
  int64_t n_solvent;
  uint64_t seed;
  int64_t init_count[4];     /* initial number of particles per species code (init) */
  double mass[4];            /* solvent mass per species code                       */
  double eps_c[4];           /* LJ epsilon, species code vs C sphere                */
  double eps_n[4];           /* LJ epsilon, species code vs N sphere                */
  double rc, rn, dcn;        /* sphere LJ radii and bond length                     */
  double mc, mn;             /* sphere masses                                       */
  double rw, ew;             /* sphere-wall LJ 9-3 parameters                       */
  double rm_delta, em;       /* motor-motor LJ extra distance and epsilon           */
  double rp_ab, rp_ba;       /* catalytic conversion probabilities                  */
  double kT, skin, rot_angle, md_dt, mpc_dt;
  double k[6];               /* bulk rate constants                                 */
  int32_t engine_only[2];    /* (precision, shell_capacity of the engine config)    */
  /* rotational_code variants (2d_array, linear_periodic_ci) */
  int32_t variant;           /* ORC_VARIANT_*                                       */
  int32_t layout;            /* ORC_LAYOUT_*: dimer placement of orc_initial        */
  int32_t layout_rows, layout_cols;  /* numrows, numcols of the grid layout         */
  int32_t owner_tags;        /* 1: B particles carry the motor that made them and
                                act as A on every other motor (type_B of
                                linear_periodic_no_ci/forces_mod.f95:79-121)     */
  int32_t reserved;
  double tether_k, tether_z; /* k_harm and zdimeq of the harmonic z tether          */
  double layout_sep;         /* sep: gap between neighbouring motors of a layout    */
} orc_params;

typedef struct orc_obs {
  double momentum[3];        /* solvent + dimer total momentum                      */
  double solvent_momentum[3];
  double kinetic_solvent, kinetic_dimer, potential;
  int64_t species_count[4];
  int64_t n_inside, n_pairs;
  int32_t time_count, time_penetrate;
  int64_t cstep;
} orc_obs;

typedef struct orc orc_t;

orc_t* orc_create(const orc_params* p);
void orc_destroy(orc_t* o);
int orc_status(const orc_t* o);
int orc_set_threads(int n);

/* RNG selection: contract (Philox, default) or MT19937 serial reference order. */
int orc_set_rng(orc_t* o, int mode, uint32_t mt_seed);
int orc_set_list_mode(orc_t* o, int mode);

/* State exchange.  Dimer arrays hold n_dimers*2 spheres (s = 2k+i) x 3 comps. */
int orc_set_state(orc_t* o, const double* x, const double* y, const double* z,
                  const double* vx, const double* vy, const double* vz,
                  const int32_t* flag, const double* dpos, const double* dvel,
                  const double* dforce);
int orc_get_state(const orc_t* o, double* x, double* y, double* z,
                  double* vx, double* vy, double* vz, int32_t* flag,
                  double* dpos, double* dvel, double* dforce);
/* Rotor anchors (motorCM) [n_dimers*3].  orc_set_state and orc_initial set
 * them to the midpoints of the dimers they receive or place. */
int orc_set_anchors(orc_t* o, const double* anchors);
int orc_get_anchors(const orc_t* o, double* anchors);
/* Owner tags (type_B): 1-based motor number of the C sphere that made a B
 * particle, 0 for none; [n_solvent].  orc_set_state and orc_initial clear them. */
/* restart_mod.f95:415-528: after orc_prepare, evaluate the forces of the
 * state (pair forces for the first half kick, catalysis, sphere totals). */
int orc_restart_forces(orc_t* o);
int orc_set_owner(orc_t* o, const int32_t* owner);
int orc_get_owner(const orc_t* o, int32_t* owner);
int orc_set_cell_order(orc_t* o, const int32_t* order, int64_t n);
int orc_set_cstep(orc_t* o, int64_t cstep, int32_t time_count);

/* Collective-driver pieces (main_pattern.f95 and the modules it calls). */
int orc_initial(orc_t* o);           /* initial_mod.f95:6-355                       */
int orc_prepare(orc_t* o);           /* main_pattern.f95:168-187                    */
int orc_step(orc_t* o);              /* main_pattern.f95:203-225 (one iteration)    */
int orc_run(orc_t* o, int64_t nsteps);
int orc_sort(orc_t* o);              /* sort_hilbert_mod.f95:6-98                   */
int orc_rebuild_lists(orc_t* o);     /* neighbour_list_mod.f95:6-184                */
int orc_distribute(orc_t* o);        /* distribute_mod.f95 / Affected_Cell.f90      */
int orc_mpc_rotation(orc_t* o);      /* mpc_rotation_mod.f95:6-239                  */
int orc_reaction(orc_t* o);          /* reaction_mod.f95:8-66 / RMPC:127-324         */

/* Faithful selkov_code driver (Main_SelkovDimer.f90:125-149). */
int orc_selkov_prepare(orc_t* o);
int orc_selkov_step(orc_t* o);

/* Inspection. */
int orc_observables(const orc_t* o, orc_obs* out);
/* Concentration fields of species 0 and 1 (output_mod.f95:482-575) from host
 * arrays: box[3]; prm = x_slab, y_slab, z_slab, half_width, x_width, y_width,
 * z_width; outputs as mpcmd_concentration (any may be NULL). */
int orc_concentration(int64_t n, const double* x, const double* y, const double* z,
                      const int32_t* flag, const double* box, const double* prm, double* totals,
                      double* c1d_a, double* c1d_b, double* xy_a, double* xy_b,
                      double* xz_a, double* xz_b, double* yz_a, double* yz_b);
int64_t orc_n_cells_shifted(const orc_t* o);
int orc_get_new_cell(const orc_t* o, int64_t* newcell);
int orc_get_cell_rotation(const orc_t* o, double* cm, double* axis, int32_t* count);
int orc_get_distribute(const orc_t* o, int32_t* counts, int64_t* first);
int orc_get_affected(const orc_t* o, int32_t* affected);
int orc_get_shift(const orc_t* o, double* shift);
int64_t orc_neighbour_count(const orc_t* o, int sphere);
int orc_get_neighbours(const orc_t* o, int sphere, int64_t* idx);
int orc_get_inside(const orc_t* o, int64_t* n_in, int64_t* idx);
int orc_get_pair_forces(const orc_t* o, int sphere, double* f, double* pot);
int orc_reactive_grid_table(const orc_t* o, int32_t* table);

/* RNG known-answer exports. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double orc_contract_u01(uint64_t seed, uint32_t tag, uint32_t index,
                        uint32_t extra, uint32_t step, int which);
void orc_mt1998_sgrnd(uint32_t seed, uint32_t* state624);
void orc_mt2002_init(uint32_t seed, uint32_t* state624);
void orc_mt_next_u32(uint32_t* state624, int32_t* mti, uint32_t* out, int64_t n);
double orc_mt_grnd(uint32_t* state624, int32_t* mti);
double orc_mt_real1(uint32_t* state624, int32_t* mti);

#ifdef __cplusplus
}
#endif
#endif
