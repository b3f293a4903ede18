// Device state of one mpcmd context and the kernel launchers the host
// orchestration in mpcmd_engine.cu drives.
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>
#include "mpcmd_device.cuh"

namespace mpcmd {

constexpr int TPB = 256;           // threads per block of the grid-stride kernels
constexpr int SHELL_CLASSES = 3;   // pair classes of the shell ordering (k_shell_hist)

// Error bits accumulated on the device (mapped to mpcmd_status on the host).
enum : int {
  DEV_ERR_CELL_OVERFLOW = 1 << 0,
  DEV_ERR_SHELL_OVERFLOW = 1 << 1,
  DEV_ERR_PAIR_OVERFLOW = 1 << 2,
  DEV_ERR_BIN_OVERFLOW = 1 << 3,
  DEV_ERR_RATTLE = 1 << 4,
  DEV_ERR_INIT = 1 << 5,
  DEV_ERR_PASSIVE = 1 << 6,   // a free-flight shell member was found inside an LJ cutoff
};

struct Counters {
  unsigned int n_inside;          // entries of the current shell buffer
  unsigned int n_inside_new;      // entries written by a running rebuild
  unsigned long long maxv2;       // bits of max v^2 (double) over all particles at a rebuild
  unsigned long long maxmsd[2];   // bits of max max_solvent_dist (double), by step parity
  int status;                     // DEV_ERR_* bits
  int abort_step;                 // step at which a displacement-triggered rebuild is due
  int time_penetrate;
  int pad;
  unsigned long long rattle_iters;
  double sums[16];                // observable reductions
  int dbg_code;                   // checked builds: first failed bounds check
  int dbg_pad;
  long long dbg_val;
  unsigned long long vsph;        // bits of the largest sphere speed seen (double)
  unsigned long long vlast;       // bits of max v^2 over all particles at the last rebuild
  unsigned long long vpost;       // bits of max v^2 of the outside particles after the last collision
  unsigned long long vfar;        // bits of max v^2 of the particles off the watch list
  unsigned int n_watch;           // entries of the watch list
  unsigned int n_near;            // particles the far pass of a collision rebuild deferred
  // work totals for the measurement (cleared by mpcmd_profile(ctx, 1))
  unsigned long long acc_force;   // shell entries over all k_force launches
  unsigned long long acc_rebuild; // particles visited over all k_rebuild launches
  unsigned long long acc_placed;  // shell entries written by the rebuilds
};

// Bounds check of the checked build (MPCMD_CHECKED): records the first failing
// check and lets the caller skip the access.  Compiles to `true` otherwise.
__device__ __forceinline__ bool chk(bool ok, Counters* c, int code, long long v) {
#ifdef MPCMD_CHECKED
  if (!ok && atomicCAS(&c->dbg_code, 0, code) == 0) c->dbg_val = v;
  return ok;
#else
  (void)c; (void)code; (void)v;
  return true;
#endif
}

template <typename T>
struct Shell {
  uint32_t* idx;       // slot of the member in the main arrays
  uint32_t* mid;       // its main index (the slot until a re-sort moves particles)
  uint32_t* cell;
  T *ox, *oy, *oz, *vx, *vy, *vz;
  T* msd;              // max_solvent_dist
  uint8_t* flag;       // species bits | FLAG_INLIST
  uint8_t* nonbulk;    // within the LJ cutoff of a sphere at the rebuild
  uint8_t* np;         // number of sphere pairs
  uint16_t* sph;       // [cap * PAIRMAX] sphere ids, ascending
  T* pf;               // [cap * PAIRMAX * 3] pair forces kept across a step boundary
  uint32_t* skey;      // shifted collision cell at an MPC step
  int64_t cap;
};

template <typename T>
struct Particles {
  uint32_t* cell;
  T *ox, *oy, *oz, *vx, *vy, *vz;
  uint8_t* flag;
};

// Concentration-field counting (mpcmd_concentration): slab centres, half
// thickness, bin widths, bin counts per axis and the device count arrays.
struct ConcArgs {
  double xs, ys, zs, hw, xw, yw, zw;
  int nx, ny, nz;
  uint32_t *c1a, *c1b, *xya, *xyb, *xza, *xzb, *yza, *yzb;
  unsigned long long* tot;   // [2] particles of species 0 and 1
};

template <typename T>
struct Dev {
  Particles<T> p;          // main home, reference index order
  Particles<T> p2;         // gather target of the sort
  uint32_t* skey;          // shifted collision cell per particle (MPC steps)
  Shell<T> sh;             // current shell buffer
  Shell<T> sh2;            // shell buffer being built by a rebuild
  double *dpos, *dvel, *dfrc, *dq;   // [ns*3] sphere state (FP64)
  SphereRel<T>* srel;      // [ns] sphere positions as cell + offset
  double* facc;            // [ns*4] -sum F_pair (xyz) and sum of pair potentials
  double* fmot;            // [ns*4] motor-motor force and potential (j < k part)
  double* anchor;          // [nd*3] rotor anchors (motorCM)
  uint16_t *owner, *owner2;  // [n] owner tags type_B by main index (null without owner_tags); sort buffer
  uint8_t *inc, *inc2;     // [n] inside a C cutoff at the last force evaluation, by main index
                           // (catalysis on exit only, else null); sort buffer
  // Order-only re-sorts move particles between slots without renumbering
  // them: lid[slot] is the particle's main index (the index the reference's
  // arrays hold it at), lpos[index] its slot.  Both null while every slot
  // holds the particle of the same index (after upload, initial and every
  // sort of the reference); lid2 is the re-sort's gather target.
  uint32_t *lid, *lid2, *lpos;
  double* dpot;            // [nd] potential of each dimer at the last force evaluation
  uint32_t* bin_cnt;       // [nbins]
  uint32_t* bin_mask;      // [ceil(nbins / 32)] bit b set: bin b lists a sphere
  uint16_t* bin_list;      // [nbins * BIN_SLOTS]
  void* acc;               // [ncell_shift] float4 (FP32) or double4 (FP64): n, sum v
  T* rot;                  // [ncell_shift * 6] centre-of-mass velocity and axis
  uint32_t* dcnt;          // [ncell] packed per-species counts (8 bits each)
  uint32_t* dfirst;        // [ncell * 4] first member key per species (dist_key)
  uint8_t* affected;       // [ncell]
  uint8_t* react_box;      // [lx*ly]
  uint32_t* order_rank;    // [ncell] position of each cell in the sort order
  uint32_t* watch;         // [n] particles that can come near a sphere or a wall before the next collision
  uint32_t* gapf;          // [nbins] bits of a lower bound on (distance to a sphere - list radius), >= 0
  uint32_t* sph_cnt;       // [ns * 3] shell entries per (first sphere, pair class) (shell ordering)
  uint32_t* sph_base;      // [ns * 3] first slot of each bucket's entries
  uint32_t* scnt;          // [ncell] sort scratch
  uint32_t* sstart;        // [ncell]
  uint32_t* sfill;         // [ncell]
  uint32_t* sidx;          // [n]
  uint32_t* scan_tmp;      // scan scratch
  Counters* ctr;
  double* staging;         // host-exchange staging [n]
  double* staging2;        // second staging buffer (copies overlap conversions)
  int32_t* staging_i;      // [n]
};

// Step-level launch arguments.
struct StepArgs {
  uint32_t step;       // cstep of the step being executed
  int tc;              // time_count: steps since the last rebuild
  int tc_full;         // steps since the last full pass (lag of deferred main-home states)
  int full;            // rebuild pass writes every particle (collision steps, sorts, prepare)
  int mpc;             // this step ends with a collision
  int advance;         // fuse kick1 + stream of the next step
  int rebuilt;         // a rebuild ran in this step
  int forces_only;     // k_force: pair forces, catalysis and sphere sums without the kicks (a restart)
  int merge_only;      // rebuild pass: lazy-stream and merge only, no lists
  int grid;            // persistent grid size of the light kernels
  int g_rebuild;       // SMs x resident blocks of k_rebuild, k_force, k_rotate_main
  int g_force;
  int g_rotate;
  int g_far;           // SMs x resident blocks of k_rebuild_far
  int g_cells;         // SMs x resident blocks of k_cells (one wave)
  int g_shell;         // SMs x resident blocks of k_shell_advance (one wave)
  int watch_build;     // > 0 (the period in steps): rotate_main / rotate_shell build the watch list
  int use_watch;       // a rebuild between full passes visits the watch list only
  int near;            // the rebuild visits the particles the far pass deferred (list in `watch`)
  int horizon;         // > 0: steps to the next collision rebuild; shell members that
                       // cannot reach an LJ cutoff or a wall before it fly freely
  double shift[3];     // collision grid shift of this step
  float shf[3];        // the same rounded to float (FP32 kernels)
};

template <typename T>
struct Launch {
  // conversion of one uploaded FP64 component (0-2 positions, 3-5
  // velocities) or of the int32 flags from a staging buffer
  static void upload_comp(const Dev<T>& d, const KParams<T>& kp, const double* src, int comp, cudaStream_t st);
  static void upload_flag(const Dev<T>& d, const KParams<T>& kp, const int32_t* src, cudaStream_t st);
  static void download_convert(const Dev<T>& d, const KParams<T>& kp, double* out, int comp, int tc,
                               int tc_defer, int current, cudaStream_t st);
  static void download_flag(const Dev<T>& d, const KParams<T>& kp, int32_t* out, int tc, int tc_defer,
                            int current, cudaStream_t st);
  static void update_srel(const Dev<T>& d, const KParams<T>& kp, cudaStream_t st);
  // tc_defer > 0: bins also reach every sphere that a deferred particle,
  // stored tc_defer steps ago, can be near now (for the rebuild fast path)
  static void build_bins(const Dev<T>& d, const KParams<T>& kp, int tc_defer, cudaStream_t st);
  static void rebuild(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st);
  // collision-step full pass split in two: a lean pass over the particles
  // whose (streamed) bin lists no sphere, which defers the others (and the
  // shell-buffer states) to a list; then k_rebuild over that list
  static void rebuild_split(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st);
  static void finalize_rebuild(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, double skin, cudaStream_t st);
  static void force(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st);
  // kick + free flight of the shell; with a.horizon > 0 it also moves the
  // free-flight members to the main home and compacts the rest into d.sh2
  // (the caller then swaps d.sh and d.sh2)
  static void advance(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st);
  static void sphere_totals(const Dev<T>& d, const KParams<T>& kp, double w3, cudaStream_t st);
  static void dimer(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, int mode,
                    double w3, int rattle_max, cudaStream_t st);
  static void affected(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st);
  static void accumulate_main(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, int what, cudaStream_t st);
  static void cells(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, int what, cudaStream_t st);
  static void rotate_main(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st);
  // lower bounds of the distance of each bin to the spheres' list radius (for the watch list)
  static void gap_field(const Dev<T>& d, const KParams<T>& kp, int horizon, cudaStream_t st);
  // order the shell entries of d.sh2 by their first sphere into d.sh (so that
  // a warp's particles share spheres); skipped when a displacement abort is pending
  static void sort_shell(const Dev<T>& d, const KParams<T>& kp, cudaStream_t st);
  static void rotate_shell(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st);
  static void flush(const Dev<T>& d, const KParams<T>& kp, cudaStream_t st);
  static void regather(const Dev<T>& d, const KParams<T>& kp, cudaStream_t st);
  static void sort(Dev<T>& d, const KParams<T>& kp, cudaStream_t st);
  // order-only re-sort: particles grouped by the sort rank of their stored
  // cell (any order inside a cell), main indices kept in lid / lpos; the
  // caller provides lid2 and lpos and swaps nothing
  static void resort(Dev<T>& d, const KParams<T>& kp, int tc, int tc_full, cudaStream_t st);
  static void observables(const Dev<T>& d, const KParams<T>& kp, const double* mass, int grid, cudaStream_t st);
  static void concentration(const Dev<T>& d, const KParams<T>& kp, int tc, int tc_defer, const ConcArgs& c,
                            cudaStream_t st);
  // resident blocks per SM of the persistent kernels (rebuild, force, rotate)
  static void occupancy(int* blocks);
  static void init_solvent(const Dev<T>& d, const KParams<T>& kp, const int64_t* bounds, double kT,
                           const double* mass, cudaStream_t st);
};

int debug_sync(cudaStream_t st, const char* where, int line);
// The engine's default cell order of the sort: cells ranked along a Hilbert
// curve of the box (order[k] = row-major id of the k-th cell).
std::vector<int32_t> default_cell_order(int lx, int ly, int lz);
void scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* tmp, cudaStream_t st);
int64_t scan_tmp_words(int64_t n);
extern int64_t g_kernel_launches;

}  // namespace mpcmd
