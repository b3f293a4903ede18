// Host orchestration and C ABI of the mpcmd engine (include/mpcmd.h).
//
// One context = one CUDA stream on the current device and one resident copy
// of the run state.  The step schedule follows main_pattern.f95:203-225 and
// evolve_mod.f95:6-732; see mpcmd_kernels.cu for the kernels.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "mpcmd.h"
#include "mpcmd_engine.cuh"

using namespace mpcmd;

namespace mpcmd {

// Hilbert index of a 3-D point (Skilling, "Programming the Hilbert curve",
// AIP Conf. Proc. 707, 2004): axes -> transpose form, then bit interleave.
uint64_t hilbert_index(uint32_t x, uint32_t y, uint32_t z, int bits) {
  uint32_t X[3] = {x, y, z};
  const int n = 3;
  uint32_t M = 1u << (bits - 1), P, Q, t;
  for (Q = M; Q > 1; Q >>= 1) {
    P = Q - 1;
    for (int i = 0; i < n; i++) {
      if (X[i] & Q) X[0] ^= P;
      else { t = (X[0] ^ X[i]) & P; X[0] ^= t; X[i] ^= t; }
    }
  }
  for (int i = 1; i < n; i++) X[i] ^= X[i - 1];
  t = 0;
  for (Q = M; Q > 1; Q >>= 1)
    if (X[n - 1] & Q) t ^= Q - 1;
  for (int i = 0; i < n; i++) X[i] ^= t;
  uint64_t h = 0;
  for (int b = bits - 1; b >= 0; --b)
    for (int i = 0; i < n; ++i) h = (h << 1) | ((X[i] >> b) & 1u);
  return h;
}

std::vector<int32_t> default_cell_order(int lx, int ly, int lz) {
  int m = std::max(lx, std::max(ly, lz)), bits = 1;
  while ((1 << bits) < m) ++bits;
  int64_t C = (int64_t)lx * ly * lz;
  std::vector<std::pair<uint64_t, int32_t>> keys((size_t)C);
  int64_t c = 0;
  for (int z = 0; z < lz; ++z)
    for (int y = 0; y < ly; ++y)
      for (int x = 0; x < lx; ++x, ++c) keys[(size_t)c] = {hilbert_index(x, y, z, bits), (int32_t)c};
  std::sort(keys.begin(), keys.end());
  std::vector<int32_t> order((size_t)C);
  for (int64_t k = 0; k < C; ++k) order[(size_t)k] = keys[(size_t)k].second;
  return order;
}

}  // namespace mpcmd

namespace {

const double kPi = 3.141592653589793;

// Kernel kinds of the per-launch timing (mpcmd_profile_read order).
enum {
  PROF_REBUILD = 0, PROF_FORCE = 1, PROF_DIMER = 2, PROF_CELLS = 3, PROF_ROTATE_MAIN = 4,
  PROF_SHELL_ADVANCE = 5, PROF_BINS = 6, PROF_FINALIZE = 7, PROF_SORT = 8, PROF_AFFECTED = 9,
  PROF_KINDS = 10
};

// reactive_grid_mod.f95:8-99 (1-based patch index as in the Fortran).
std::vector<uint8_t> reactive_table(const mpcmd_config& c) {
  const double b1 = c.lx, b2 = c.ly;
  const int ib1 = c.lx;
  const int64_t nbox = (int64_t)c.lx * c.ly;
  const double sixth = (double)(1.0f / 6.0f), fivesixth = (double)(5.0f / 6.0f);
  std::vector<uint8_t> t((size_t)nbox, 0);
  if (c.geometry != MPCMD_GEOM_WALLS) return t;
  for (int64_t i = 1; i <= nbox; ++i) {
    int set = 0;
    switch (c.react_box_type) {
      case 1: { int64_t m = i % ib1; set = (m > 0 && m <= (int64_t)(0.5 * b1)); break; }
      case 2: { int64_t f = (int64_t)std::floor((double)i / b2); set = ((i + f) % 2 == 0); break; }
      case 3: {
        double a = 0.5 * b1 - (double)((i - 1) % ib1) + 0.5;
        double q = 0.5 * b2 - (double)(int64_t)std::floor((double)i / b1) + 0.5;
        set = (a * a + q * q < 400.0);
        break;
      }
      case 4: {
        double xm = (double)((i - 1) % ib1), yf = (double)(int64_t)std::floor((double)i / b1);
        double cx[3] = {sixth * b1, 0.5 * b1, fivesixth * b1}, cy[2] = {0.25 * b2, 0.75 * b2};
        set = 1;
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 2; ++b) {
            double u = cx[a] - xm + 0.5, v = cy[b] - yf + 0.5;
            if (!(u * u + v * v < 100.0)) set = 0;
          }
        break;
      }
      case 5: { int64_t m = i % ib1; set = (m > (int64_t)std::floor(0.5 * b1 - 4) && m <= (int64_t)std::floor(0.5 * b1 + 4)); break; }
      case 6: set = 1; break;
      default: break;
    }
    if (set) t[(size_t)(i - 1)] = 1;
  }
  return t;
}

int dev_status_to_api(int bits) {
  if (bits & DEV_ERR_CELL_OVERFLOW) return MPCMD_ERR_CELL_OVERFLOW;
  if (bits & (DEV_ERR_SHELL_OVERFLOW | DEV_ERR_PAIR_OVERFLOW | DEV_ERR_BIN_OVERFLOW | DEV_ERR_PASSIVE))
    return MPCMD_ERR_NEIGHBOUR_OVERFLOW;
  if (bits & DEV_ERR_RATTLE) return MPCMD_ERR_RATTLE;
  if (bits & DEV_ERR_INIT) return MPCMD_ERR_INIT;
  return MPCMD_OK;
}

struct EngineBase {
  virtual ~EngineBase() {}
  virtual int init(const mpcmd_config& c) = 0;
  virtual int upload(const double* x, const double* y, const double* z, const double* vx, const double* vy,
                     const double* vz, const int32_t* flag, const double* dpos, const double* dvel,
                     const double* dforce) = 0;
  virtual int download(double* x, double* y, double* z, double* vx, double* vy, double* vz, int32_t* flag,
                       double* dpos, double* dvel, double* dforce) = 0;
  virtual int set_order(const int32_t* order, int64_t n) = 0;
  virtual int set_anchors(const double* a) = 0;
  virtual int get_anchors(double* a) = 0;
  virtual int set_owner_tags(const int32_t* t) = 0;
  virtual int get_owner_tags(int32_t* t) = 0;
  virtual int set_step(int64_t cstep, int32_t tc) = 0;
  virtual int set_collision(double rot_angle, double mpc_dt, const double* k) = 0;
  virtual int set_resort(int64_t every) = 0;
  virtual int set_reactive_grid(const int32_t* table) = 0;
  virtual int initial() = 0;
  virtual int prepare() = 0;
  virtual int prepare_restart() = 0;
  virtual int run(int64_t nsteps, bool with_mpc) = 0;
  virtual int sort_stage() = 0;
  virtual int rebuild_stage() = 0;
  virtual int distribute_stage() = 0;
  virtual int rotation_stage() = 0;
  virtual int reaction_stage() = 0;
  virtual int observables(mpcmd_obs* o) = 0;
  virtual int concentration(const mpcmd_conc_params* p, double* totals, double* const* fields) = 0;
  virtual int dimer_axes(int normalize, double* nucvec, double* vdot) = 0;
  virtual int get_new_cell(int64_t* out) = 0;
  virtual int get_cell_rotation(double* cm, double* axis, int32_t* count) = 0;
  virtual int get_distribute(int32_t* counts, int64_t* first) = 0;
  virtual int get_affected(int32_t* a) = 0;
  virtual int get_pairs(int64_t* np, int64_t* part, int32_t* sph) = 0;
  virtual int get_inside(int64_t* n, int64_t* idx) = 0;
  virtual int get_counters(int64_t* c, int32_t n) = 0;
  virtual int checkpoint(const char* path) = 0;
  virtual int restore(const char* path) = 0;
  virtual int event_record(int slot) = 0;
  virtual int event_elapsed(int a, int b, double* ms) = 0;
  virtual int synchronize() = 0;
  virtual int profile(int enable) = 0;
  virtual int profile_read(double* ms, int64_t* count, int n) = 0;
  int64_t bytes = 0;
  double shift[3] = {0, 0, 0};
  std::vector<int32_t> order;
  std::vector<uint8_t> react;
  mpcmd_config cfg;
};

#define CK(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) {                                  \
      last_cuda = e_;                                         \
      return MPCMD_ERR_CUDA;                                  \
    }                                                         \
  } while (0)

cudaError_t last_cuda = cudaSuccess;

template <typename T>
struct Engine : EngineBase {
  Dev<T> d{};
  KParams<T> kp{};
  cudaStream_t st = nullptr;
  // host exchange: copies on cst overlap the conversions on st, through two
  // staging buffers (events: copy done, conversion done, per buffer)
  cudaStream_t cst = nullptr;
  cudaEvent_t xev[4] = {nullptr, nullptr, nullptr, nullptr};
  std::vector<void*> allocs;
  int grid = 0, g_rebuild = 0, g_force = 0, g_rotate = 0, g_far = 0, g_cells = 0, g_shell = 0;
  int64_t cstep = 0;
  int time_count = 0, time_penetrate = 0;
  int64_t last_rebuild = 0;
  int64_t last_full = 0;   // step of the last rebuild that wrote every particle
  int64_t force_rebuild_step = -1;
  bool prepared = false, home_shell = false, advanced = false;
  // the next prepare evaluates the forces of the state, as restart_mod.f95 does
  bool restart_pending = false;
  // the watch list of the last collision is valid (no full pass or stage call since)
  bool watch_valid = false;
  // order-only re-sort every resort_every MD steps (a multiple of the
  // collision interval; 0 = never): two slot -> index buffers and the
  // index -> slot table
  int64_t resort_every = 0, resorts = 0;
  uint32_t *lid_a = nullptr, *lid_b = nullptr, *lpos_buf = nullptr;
  double w3 = 1.0;
  unsigned int n_inside = 0;

  // ---- measurement: named stream events and per-kernel launch timing ----
  cudaEvent_t marks[8] = {};
  bool profiling = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_open;
  std::vector<cudaEvent_t> prof_pool;
  double prof_ms[PROF_KINDS] = {};
  int64_t prof_n[PROF_KINDS] = {};

  cudaEvent_t pool_get() {
    if (!prof_pool.empty()) { cudaEvent_t e = prof_pool.back(); prof_pool.pop_back(); return e; }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  void pb(int kind) {
    if (!profiling) return;
    cudaEvent_t a = pool_get(), b = pool_get();
    cudaEventRecord(a, st);
    prof_open.push_back({kind, {a, b}});
  }
  void pe() {
    if (!profiling || prof_open.empty()) return;
    cudaEventRecord(prof_open.back().second.second, st);
  }
  void prof_collect() {
    cudaStreamSynchronize(st);
    for (auto& r : prof_open) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, r.second.first, r.second.second);
      prof_ms[r.first] += ms;
      prof_n[r.first] += 1;
      prof_pool.push_back(r.second.first);
      prof_pool.push_back(r.second.second);
    }
    prof_open.clear();
  }

  ~Engine() override {
    if (st) cudaStreamSynchronize(st);
    for (auto& r : prof_open) { cudaEventDestroy(r.second.first); cudaEventDestroy(r.second.second); }
    for (cudaEvent_t e : prof_pool) cudaEventDestroy(e);
    for (cudaEvent_t e : marks) if (e) cudaEventDestroy(e);
    if (cst) cudaStreamSynchronize(cst);
    for (cudaEvent_t e : xev) if (e) cudaEventDestroy(e);
    for (void* p : allocs) cudaFree(p);
    if (cst) cudaStreamDestroy(cst);
    if (st) cudaStreamDestroy(st);
  }

  template <typename U>
  int alloc(U*& p, int64_t count) {
    size_t b = (size_t)std::max<int64_t>(count, 1) * sizeof(U);
    void* q = nullptr;
    if (cudaMalloc(&q, b) != cudaSuccess) { cudaGetLastError(); return MPCMD_ERR_ALLOC; }
    allocs.push_back(q);
    bytes += (int64_t)b;
    p = (U*)q;
    return MPCMD_OK;
  }

  int alloc_particles(Particles<T>& p, int64_t n) {
    int r = 0;
    r |= alloc(p.cell, n);
    r |= alloc(p.ox, n); r |= alloc(p.oy, n); r |= alloc(p.oz, n);
    r |= alloc(p.vx, n); r |= alloc(p.vy, n); r |= alloc(p.vz, n);
    r |= alloc(p.flag, n);
    return r ? MPCMD_ERR_ALLOC : MPCMD_OK;
  }

  int alloc_shell(Shell<T>& s, int64_t cap) {
    int r = 0;
    s.cap = cap;
    r |= alloc(s.idx, cap); r |= alloc(s.mid, cap); r |= alloc(s.cell, cap);
    r |= alloc(s.ox, cap); r |= alloc(s.oy, cap); r |= alloc(s.oz, cap);
    r |= alloc(s.vx, cap); r |= alloc(s.vy, cap); r |= alloc(s.vz, cap);
    r |= alloc(s.msd, cap); r |= alloc(s.flag, cap); r |= alloc(s.nonbulk, cap); r |= alloc(s.np, cap);
    r |= alloc(s.sph, cap * PAIRMAX); r |= alloc(s.pf, cap * PAIRMAX * 3); r |= alloc(s.skey, cap);
    return r ? MPCMD_ERR_ALLOC : MPCMD_OK;
  }

  int init(const mpcmd_config& c) override {
    cfg = c;
    if (c.lx <= 0 || c.ly <= 0 || c.lz <= 0 || c.lx > 1024 || c.ly > 1024 || c.lz > 1023) return MPCMD_ERR_CONFIG;
    if (c.n_solvent <= 0 || c.n_solvent >= (int64_t)1 << 31 || c.n_dimers < 0 || 2 * c.n_dimers > 65535)
      return MPCMD_ERR_CONFIG;
    if (c.mpc_every <= 0 || c.md_dt <= 0 || c.cell_capacity <= 0 || c.cell_capacity > 255) return MPCMD_ERR_CONFIG;
    if (c.kinetics == MPCMD_KIN_SELKOV && c.geometry != MPCMD_GEOM_PERIODIC) return MPCMD_ERR_CONFIG;
    if (c.variant != MPCMD_VARIANT_MOTOR && c.variant != MPCMD_VARIANT_ROTOR) return MPCMD_ERR_CONFIG;
    if (c.catalysis < MPCMD_CAT_DETERMINISTIC || c.catalysis > MPCMD_CAT_ON_EXIT) return MPCMD_ERR_CONFIG;
    if (c.variant == MPCMD_VARIANT_ROTOR && !(c.tether_k >= 0.0)) return MPCMD_ERR_CONFIG;
    if (c.owner_tags != 0 &&
        (c.owner_tags != 1 || c.catalysis != MPCMD_CAT_DETERMINISTIC || c.kinetics == MPCMD_KIN_SELKOV ||
         (c.geometry == MPCMD_GEOM_WALLS && c.react_box_type >= 1 && c.react_box_type <= 6)))
      return MPCMD_ERR_CONFIG;
    if (c.layout == MPCMD_LAYOUT_GRID ? (c.layout_rows <= 0 || c.layout_cols <= 0 ||
                                         (int64_t)c.layout_rows * c.layout_cols != c.n_dimers)
                                      : (c.layout != MPCMD_LAYOUT_RANDOM && c.layout != MPCMD_LAYOUT_LINE))
      return MPCMD_ERR_CONFIG;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    grid = nsm * 8;
    // the heavy persistent kernels run exactly one wave: SMs x resident blocks
    int occ[6];
    Launch<T>::occupancy(occ);
    CK(cudaGetLastError());
    g_rebuild = nsm * std::max(occ[0], 1);
    g_force = nsm * std::max(occ[1], 1);
    g_rotate = nsm * std::max(occ[2], 1);
    g_far = nsm * std::max(occ[3], 1);
    g_cells = nsm * std::max(occ[4], 1);
    g_shell = nsm * std::max(occ[5], 1);
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&cst, cudaStreamNonBlocking));
    for (cudaEvent_t& e : xev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));

    const int64_t n = c.n_solvent, ns = 2 * (int64_t)c.n_dimers;
    kp.lx = c.lx; kp.ly = c.ly; kp.lz = c.lz;
    kp.geometry = c.geometry; kp.ns = (int)ns; kp.nd = c.n_dimers;
    kp.catalysis = c.catalysis; kp.exclusion = c.exclusion; kp.kinetics = c.kinetics;
    kp.rotation_sense = c.rotation_sense >= 0 ? 1 : -1;
    kp.react_dir = c.react_dir; kp.cell_capacity = c.cell_capacity;
    kp.n = n;
    kp.ncell = (int64_t)c.lx * c.ly * c.lz;
    kp.ncell_shift = c.geometry == MPCMD_GEOM_WALLS ? (int64_t)c.lx * c.ly * (c.lz + 1) : kp.ncell;
    kp.seed = c.seed;
    kp.Lx = (T)c.lx; kp.Ly = (T)c.ly; kp.Lz = (T)c.lz;
    kp.Ld[0] = c.lx; kp.Ld[1] = c.ly; kp.Ld[2] = c.lz;
    kp.dt = (T)c.md_dt; kp.dtd = c.md_dt;
    for (int s = 0; s < 4; ++s) {
      kp.hIM[s] = (T)((0.5 * c.md_dt) / (c.mass[s] > 0 ? c.mass[s] : 1.0));
      kp.eps_c[s] = (T)c.eps_c[s];
      kp.eps_n[s] = (T)c.eps_n[s];
    }
    const double cut = std::pow(2.0, 1.0 / 6.0);
    const double R[2] = {c.rc, c.rn};
    for (int t = 0; t < 2; ++t) {
      double co = R[t] * cut;
      kp.cut2[t] = (T)(co * co);
      kp.cut2_strict[t] = (T)(co * co);
      kp.full2[t] = (T)((co + c.skin) * (co + c.skin));
      double r2 = R[t] * R[t], R6 = r2 * r2 * r2, R12 = R6 * R6;
      kp.R6[t] = (T)R6; kp.R12[t] = (T)R12; kp.r6R6[t] = (T)(6.0 * R6); kp.r12R12[t] = (T)(12.0 * R12);
    }
    kp.msd_thr = (T)((0.5 * c.skin) * (0.5 * c.skin));
    kp.cosrot = (T)std::cos(c.rot_angle);
    kp.sinrot = (T)std::sin(c.rot_angle);
    kp.rp_ab = c.rp_ab; kp.rp_ba = c.rp_ba;
    kp.thr_ab = prob_threshold(c.rp_ab);
    kp.thr_ba = prob_threshold(c.rp_ba);
    kp.tau = c.mpc_dt;
    for (int q = 0; q < 6; ++q) { kp.k[q] = c.k[q]; kp.kf[q] = (float)c.k[q]; }
    kp.tauf = (float)c.mpc_dt;
    kp.nbx = (c.lx + BIN_EDGE - 1) / BIN_EDGE;
    kp.nby = (c.ly + BIN_EDGE - 1) / BIN_EDGE;
    kp.nbz = (c.lz + BIN_EDGE - 1) / BIN_EDGE;
    kp.ngx = (c.lx + GAP_EDGE - 1) / GAP_EDGE;
    kp.ngy = (c.ly + GAP_EDGE - 1) / GAP_EDGE;
    kp.ngz = (c.lz + GAP_EDGE - 1) / GAP_EDGE;
    const double msum[3] = {c.rc + c.rc + c.rm_delta, c.rc + c.rn + c.rm_delta, c.rn + c.rn + c.rm_delta};
    for (int t = 0; t < 3; ++t) {
      double r2 = msum[t] * msum[t], R6 = r2 * r2 * r2, R12 = R6 * R6;
      kp.mot_cut2[t] = (msum[t] * cut) * (msum[t] * cut);
      kp.mot_cut2f[t] = (float)kp.mot_cut2[t];
      kp.mot_R6[t] = R6; kp.mot_R12[t] = R12; kp.mot_r6R6[t] = 6.0 * R6; kp.mot_r12R12[t] = 12.0 * R12;
    }
    kp.em = c.em; kp.ew = c.ew; kp.rwc = c.rw + c.rc; kp.rwn = c.rw + c.rn;
    kp.rotor = c.variant == MPCMD_VARIANT_ROTOR ? 1 : 0;
    kp.owner_tags = c.owner_tags;
    kp.tether_k = c.tether_k; kp.tether_z = c.tether_z;
    kp.mc = c.mc; kp.mn = c.mn; kp.dcn = c.dcn;
    kp.hIMc = (0.5 * c.md_dt) / c.mc; kp.hIMn = (0.5 * c.md_dt) / c.mn;
    kp.IIM = 1.0 / ((1.0 / c.mc) + (1.0 / c.mn));
    kp.iMc = 1.0 / c.mc; kp.iMn = 1.0 / c.mn; kp.iD2 = 1.0 / (c.dcn * c.dcn);
    kp.iMcdt = 1.0 / (c.mc * c.md_dt); kp.iMndt = 1.0 / (c.mn * c.md_dt);
    w3 = std::pow(3.0, (double)(1.0f / 6.0f));

    // shell capacity from the sphere shells
    int64_t cap = c.shell_capacity;
    if (cap <= 0) {
      double rho = (double)n / (double)kp.ncell;
      double vc = 4.0 / 3.0 * kPi * std::pow(c.rc * cut + c.skin + 1.0, 3);
      double vn = 4.0 / 3.0 * kPi * std::pow(c.rn * cut + c.skin + 1.0, 3);
      double est = 2.0 * (double)c.n_dimers * (vc + vn) * rho * 1.5 + 8192.0;
      cap = (int64_t)std::min<double>((double)n, est);
    }
    int r = 0;
    r |= alloc_particles(d.p, n);
    r |= alloc_particles(d.p2, n);
    r |= alloc(d.skey, n);
    r |= alloc(d.sidx, n);
    r |= alloc(d.staging, n);
    r |= alloc(d.staging2, n);
    r |= alloc(d.staging_i, n);
    r |= alloc_shell(d.sh, cap);
    r |= alloc_shell(d.sh2, cap);
    const int64_t ns1 = std::max<int64_t>(ns, 1), nd1 = std::max<int64_t>(c.n_dimers, 1);
    r |= alloc(d.dpos, 3 * ns1); r |= alloc(d.dvel, 3 * ns1); r |= alloc(d.dfrc, 3 * ns1); r |= alloc(d.dq, 3 * ns1);
    r |= alloc(d.srel, ns1); r |= alloc(d.facc, 4 * ns1); r |= alloc(d.fmot, 4 * ns1); r |= alloc(d.dpot, nd1);
    int64_t nbins = (int64_t)kp.nbx * kp.nby * kp.nbz;
    r |= alloc(d.bin_cnt, nbins); r |= alloc(d.bin_list, nbins * BIN_SLOTS);
    r |= alloc(d.bin_mask, (nbins + 31) / 32);
    r |= alloc(d.gapf, (int64_t)kp.ngx * kp.ngy * kp.ngz); r |= alloc(d.watch, n);
    r |= alloc(d.sph_cnt, ns1 * SHELL_CLASSES); r |= alloc(d.sph_base, ns1 * SHELL_CLASSES);
    if (sizeof(T) == 4) { float4* a = nullptr; r |= alloc(a, kp.ncell_shift); d.acc = a; }
    else { double* a = nullptr; r |= alloc(a, 4 * kp.ncell_shift); d.acc = a; }
    r |= alloc(d.rot, 6 * kp.ncell_shift);
    r |= alloc(d.dcnt, kp.ncell); r |= alloc(d.dfirst, 4 * kp.ncell); r |= alloc(d.affected, kp.ncell);
    r |= alloc(d.react_box, (int64_t)c.lx * c.ly);
    r |= alloc(d.order_rank, kp.ncell);
    int64_t cmax = std::max(kp.ncell, kp.ncell_shift);
    r |= alloc(d.scnt, cmax); r |= alloc(d.sstart, kp.ncell); r |= alloc(d.sfill, kp.ncell);
    r |= alloc(d.scan_tmp, scan_tmp_words(kp.ncell));
    r |= alloc(d.ctr, 1);
    // (the variant arrays last: the allocations above keep their placement)
    r |= alloc(d.anchor, 3 * nd1);
    if (c.owner_tags) { r |= alloc(d.owner, n); r |= alloc(d.owner2, n); }
    if (c.catalysis == MPCMD_CAT_ON_EXIT) { r |= alloc(d.inc, n); r |= alloc(d.inc2, n); }
    r |= alloc(lid_a, n); r |= alloc(lid_b, n); r |= alloc(lpos_buf, n);
    if (r) return MPCMD_ERR_ALLOC;
    d.lid = d.lid2 = d.lpos = nullptr;
    // a re-sort every ten collision periods (the cell order of a diffusing
    // solvent decays within a few periods; a re-sort costs about one pass)
    resort_every = c.mpc_every > 0 ? 10 * (int64_t)c.mpc_every : 0;

    CK(cudaMemsetAsync(d.acc, 0, (sizeof(T) == 4 ? 16 : 32) * (size_t)kp.ncell_shift, st));
    CK(cudaMemsetAsync(d.dcnt, 0, 4 * (size_t)kp.ncell, st));
    CK(cudaMemsetAsync(d.dfirst, 0xFF, 16 * (size_t)kp.ncell, st));
    CK(cudaMemsetAsync(d.affected, 0, (size_t)kp.ncell, st));
    CK(cudaMemsetAsync(d.ctr, 0, sizeof(Counters), st));
    CK(cudaMemsetAsync(d.facc, 0, sizeof(double) * 4 * std::max<int64_t>(ns, 1), st));
    CK(cudaMemsetAsync(d.fmot, 0, sizeof(double) * 4 * std::max<int64_t>(ns, 1), st));
    CK(cudaMemsetAsync(d.dq, 0, sizeof(double) * 3 * std::max<int64_t>(ns, 1), st));
    CK(cudaMemsetAsync(d.anchor, 0, sizeof(double) * 3 * (size_t)nd1, st));
    if (d.owner) CK(cudaMemsetAsync(d.owner, 0, sizeof(uint16_t) * (size_t)n, st));
    if (d.inc) CK(cudaMemsetAsync(d.inc, 0, (size_t)n, st));
    CK(cudaMemsetAsync(d.p.flag, 0, (size_t)n, st));
    react = reactive_table(c);
    CK(cudaMemcpyAsync(d.react_box, react.data(), react.size(), cudaMemcpyHostToDevice, st));
    order = default_cell_order(c.lx, c.ly, c.lz);
    CK(upload_order());
    CK(cudaStreamSynchronize(st));
    return MPCMD_OK;
  }

  cudaError_t upload_order() {
    std::vector<uint32_t> rank(order.size());
    for (size_t k = 0; k < order.size(); ++k) rank[(size_t)order[k]] = (uint32_t)k;
    return cudaMemcpy(d.order_rank, rank.data(), rank.size() * 4, cudaMemcpyHostToDevice);
  }

  int set_order(const int32_t* o, int64_t n) override {
    if (n != kp.ncell) return MPCMD_ERR_CONFIG;
    std::vector<char> seen((size_t)n, 0);
    for (int64_t k = 0; k < n; ++k) {
      if (o[k] < 0 || o[k] >= n || seen[(size_t)o[k]]) return MPCMD_ERR_CONFIG;
      seen[(size_t)o[k]] = 1;
    }
    order.assign(o, o + n);
    CK(upload_order());
    return MPCMD_OK;
  }

  int set_resort(int64_t every) override {
    if (every < 0 || (every > 0 && every % cfg.mpc_every != 0)) return MPCMD_ERR_CONFIG;
    resort_every = every;
    return MPCMD_OK;
  }

  // Order-only re-sort at the start of a collision step's rebuild (the lists
  // that hold slots are rebuilt right after it; the shell learns its
  // members' new slots).
  void resort(int tc, int tc_full) {
    d.lpos = lpos_buf;
    d.lid2 = d.lid == lid_a ? lid_b : lid_a;
    Launch<T>::resort(d, kp, tc, tc_full, st);
    ++resorts;
  }

  // Main index of every slot (empty while every slot holds the particle of
  // its own index).
  int host_lid(std::vector<uint32_t>& v) {
    v.clear();
    if (!d.lid) return MPCMD_OK;
    v.resize((size_t)kp.n);
    CK(cudaMemcpyAsync(v.data(), d.lid, v.size() * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return MPCMD_OK;
  }

  // Collision angle, interval and rate constants as a driver passes them to
  // mpc_rotation / reaction_simple (mpc_rotation_mod.f95:6, reaction_mod.f95:8)
  int set_collision(double rot_angle, double mpc_dt, const double* k) override {
    if (!(mpc_dt > 0)) return MPCMD_ERR_CONFIG;
    cfg.rot_angle = rot_angle;
    cfg.mpc_dt = mpc_dt;
    kp.cosrot = (T)std::cos(rot_angle);
    kp.sinrot = (T)std::sin(rot_angle);
    kp.tau = mpc_dt;
    kp.tauf = (float)mpc_dt;
    if (k)
      for (int q = 0; q < 6; ++q) { cfg.k[q] = k[q]; kp.k[q] = k[q]; kp.kf[q] = (float)k[q]; }
    return MPCMD_OK;
  }

  // The reactive floor as the driver's react_box array (reactive_grid_mod.f95:8-99).
  int set_reactive_grid(const int32_t* table) override {
    if (!table) return MPCMD_ERR_CONFIG;
    for (size_t i = 0; i < react.size(); ++i) react[i] = table[i] ? 1 : 0;
    CK(cudaMemcpyAsync(d.react_box, react.data(), react.size(), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    return MPCMD_OK;
  }

  int set_step(int64_t c, int32_t tc) override {
    cstep = c;
    time_count = tc;
    last_rebuild = c - tc;
    last_full = last_rebuild;
    watch_valid = false;
    return MPCMD_OK;
  }

  int read_counters(Counters& h) {
    CK(cudaGetLastError());   // launch-configuration errors of the kernels queued so far
    CK(cudaMemcpyAsync(&h, d.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return MPCMD_OK;
  }

  int check_device_status() {
    Counters h;
    int r = read_counters(h);
    if (r) return r;
    n_inside = h.n_inside;
    return dev_status_to_api(h.status);
  }

  int flush_shell() {
    watch_valid = false;
    if (!home_shell) return MPCMD_OK;
    Launch<T>::flush(d, kp, st);
    home_shell = false;
    return MPCMD_OK;
  }

  int regather_shell() {
    if (home_shell || !prepared) return MPCMD_OK;
    Launch<T>::regather(d, kp, st);
    home_shell = true;
    return MPCMD_OK;
  }

  int upload(const double* x, const double* y, const double* z, const double* vx, const double* vy,
             const double* vz, const int32_t* flag, const double* dpos, const double* dvel,
             const double* dforce) override {
    // component c is copied into buffer c & 1 on cst while component c - 1 is
    // converted on st; a buffer is refilled only after its last conversion
    const double* comps[6] = {x, y, z, vx, vy, vz};
    double* buf[2] = {d.staging, d.staging2};
    cudaEvent_t copied[2] = {xev[0], xev[1]}, used[2] = {xev[2], xev[3]};
    CK(cudaEventRecord(used[0], st));
    CK(cudaEventRecord(used[1], st));
    CK(cudaStreamWaitEvent(cst, used[0], 0));
    for (int c = 0; c < 6; ++c) {
      const int b = c & 1;
      CK(cudaStreamWaitEvent(cst, used[b], 0));
      CK(cudaMemcpyAsync(buf[b], comps[c], sizeof(double) * kp.n, cudaMemcpyHostToDevice, cst));
      CK(cudaEventRecord(copied[b], cst));
      CK(cudaStreamWaitEvent(st, copied[b], 0));
      Launch<T>::upload_comp(d, kp, buf[b], c, st);
      CK(cudaEventRecord(used[b], st));
    }
    if (d.owner) CK(cudaMemsetAsync(d.owner, 0, sizeof(uint16_t) * (size_t)kp.n, st));
    if (d.inc) CK(cudaMemsetAsync(d.inc, 0, (size_t)kp.n, st));
    d.lid = d.lpos = nullptr;   // the uploaded arrays are in index order
    CK(cudaMemcpyAsync(d.staging_i, flag, sizeof(int32_t) * kp.n, cudaMemcpyHostToDevice, cst));
    CK(cudaEventRecord(copied[0], cst));
    CK(cudaStreamWaitEvent(st, copied[0], 0));
    Launch<T>::upload_flag(d, kp, d.staging_i, st);
    const size_t nb = sizeof(double) * 3 * (size_t)kp.ns;
    if (kp.ns > 0) {
      CK(cudaMemcpyAsync(d.dpos, dpos, nb, cudaMemcpyHostToDevice, st));
      CK(cudaMemcpyAsync(d.dvel, dvel, nb, cudaMemcpyHostToDevice, st));
      if (dforce) CK(cudaMemcpyAsync(d.dfrc, dforce, nb, cudaMemcpyHostToDevice, st));
      else CK(cudaMemsetAsync(d.dfrc, 0, nb, st));
      Launch<T>::update_srel(d, kp, st);
      int r = set_anchors(midpoints(dpos).data());
      if (r) return r;
    }
    CK(cudaMemsetAsync(d.ctr, 0, sizeof(Counters), st));
    CK(cudaStreamSynchronize(st));
    prepared = false; home_shell = false; advanced = false; n_inside = 0;
    restart_pending = false;
    return MPCMD_OK;
  }

  // motorCM(k,:) = 0.5 * (X(k,1) + X(k,2)) (rotational_code/2d_array/initial_mod.f95:86-88)
  std::vector<double> midpoints(const double* pos) const {
    std::vector<double> m(3 * (size_t)kp.nd);
    for (int k = 0; k < kp.nd; ++k)
      for (int q = 0; q < 3; ++q) m[3 * k + q] = 0.5 * (pos[3 * (2 * k) + q] + pos[3 * (2 * k + 1) + q]);
    return m;
  }

  int set_anchors(const double* a) override {
    if (kp.nd == 0) return MPCMD_OK;
    if (!a) return MPCMD_ERR_CONFIG;
    CK(cudaMemcpyAsync(d.anchor, a, sizeof(double) * 3 * (size_t)kp.nd, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    return MPCMD_OK;
  }

  int get_anchors(double* a) override {
    if (kp.nd == 0) return MPCMD_OK;
    if (!a) return MPCMD_ERR_CONFIG;
    CK(cudaMemcpyAsync(a, d.anchor, sizeof(double) * 3 * (size_t)kp.nd, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return MPCMD_OK;
  }

  int set_owner_tags(const int32_t* t) override {
    if (!d.owner || !t) return MPCMD_ERR_CONFIG;
    std::vector<uint32_t> lid;
    int r = host_lid(lid);
    if (r) return r;
    std::vector<uint16_t> h((size_t)kp.n);
    for (int64_t i = 0; i < kp.n; ++i) {
      const int32_t v = t[lid.empty() ? i : (int64_t)lid[(size_t)i]];
      if (v < 0 || v > kp.nd) return MPCMD_ERR_CONFIG;
      h[(size_t)i] = (uint16_t)v;
    }
    CK(cudaMemcpyAsync(d.owner, h.data(), h.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    return MPCMD_OK;
  }

  int get_owner_tags(int32_t* t) override {
    if (!d.owner || !t) return MPCMD_ERR_CONFIG;
    std::vector<uint32_t> lid;
    int r = host_lid(lid);
    if (r) return r;
    std::vector<uint16_t> h((size_t)kp.n);
    CK(cudaMemcpyAsync(h.data(), d.owner, h.size() * sizeof(uint16_t), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int64_t i = 0; i < kp.n; ++i) t[lid.empty() ? i : (int64_t)lid[(size_t)i]] = h[(size_t)i];
    return MPCMD_OK;
  }

  int download(double* x, double* y, double* z, double* vx, double* vy, double* vz, int32_t* flag,
               double* dpos, double* dvel, double* dforce) override {
    return download_state(x, y, z, vx, vy, vz, flag, dpos, dvel, dforce, false);
  }

  // `current`: every particle at the current step (a checkpoint) instead of
  // the reference's view with the outside particles at the last rebuild
  int download_state(double* x, double* y, double* z, double* vx, double* vy, double* vz, int32_t* flag,
                     double* dpos, double* dvel, double* dforce, bool current) {
    if (advanced) return MPCMD_ERR_STATE;
    flush_shell();
    // component c is converted into buffer c & 1 on st while component c - 1
    // is copied out on cst; a buffer is rewritten only after its copy
    double* outs[6] = {x, y, z, vx, vy, vz};
    double* buf[2] = {d.staging, d.staging2};
    cudaEvent_t copied[2] = {xev[0], xev[1]}, done[2] = {xev[2], xev[3]};
    CK(cudaEventRecord(copied[0], cst));
    CK(cudaEventRecord(copied[1], cst));
    int k = 0;
    for (int c = 0; c < 6; ++c) {
      if (!outs[c]) continue;
      const int b = k++ & 1;
      CK(cudaStreamWaitEvent(st, copied[b], 0));
      Launch<T>::download_convert(d, kp, buf[b], c, time_count, (int)(last_rebuild - last_full), current ? 1 : 0,
                                  st);
      CK(cudaEventRecord(done[b], st));
      CK(cudaStreamWaitEvent(cst, done[b], 0));
      CK(cudaMemcpyAsync(outs[c], buf[b], sizeof(double) * kp.n, cudaMemcpyDeviceToHost, cst));
      CK(cudaEventRecord(copied[b], cst));
    }
    if (flag) {
      Launch<T>::download_flag(d, kp, d.staging_i, time_count, (int)(last_rebuild - last_full), current ? 1 : 0,
                               st);
      CK(cudaEventRecord(done[0], st));
      CK(cudaStreamWaitEvent(cst, done[0], 0));
      CK(cudaMemcpyAsync(flag, d.staging_i, sizeof(int32_t) * kp.n, cudaMemcpyDeviceToHost, cst));
    }
    CK(cudaStreamSynchronize(cst));
    const size_t nb = sizeof(double) * 3 * (size_t)kp.ns;
    if (kp.ns > 0) {
      if (dpos) CK(cudaMemcpyAsync(dpos, d.dpos, nb, cudaMemcpyDeviceToHost, st));
      if (dvel) CK(cudaMemcpyAsync(dvel, d.dvel, nb, cudaMemcpyDeviceToHost, st));
      if (dforce) CK(cudaMemcpyAsync(dforce, d.dfrc, nb, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    return check_device_status();
  }

  StepArgs args(int64_t step) const {
    StepArgs a{};
    a.step = (uint32_t)step;
    a.grid = grid;
    a.g_rebuild = g_rebuild; a.g_force = g_force; a.g_rotate = g_rotate; a.g_far = g_far; a.g_cells = g_cells; a.g_shell = g_shell;
    a.shift[0] = shift[0]; a.shift[1] = shift[1]; a.shift[2] = shift[2];
    for (int c = 0; c < 3; ++c) a.shf[c] = (float)shift[c];
    return a;
  }

  void draw_shift(int64_t step) {
    // mpc_rotation_mod.f95:102-107 with the contract stream (SHIFT, 0, extra, step)
    double u0, u1, u2, u3;
    contract_pair(cfg.seed, TAG_SHIFT, 0, 0, (uint32_t)step, u0, u1);
    contract_pair(cfg.seed, TAG_SHIFT, 0, 1, (uint32_t)step, u2, u3);
    const double a0 = 1.0;
    shift[0] = a0 * (u0 - 0.5);
    shift[1] = a0 * (u1 - 0.5);
    shift[2] = a0 * (u2 - 0.5);
  }

  // The rebuild block of evolve_mod.f95:465-564 at step n (lazy streaming by
  // tc, optional sort, lists, time_penetrate).  Synchronises; on return the new
  // shell buffer is current.
  // Steps from step m to the next collision step (where a rebuild always
  // runs and merges the free-flight shell members back).
  int steps_to_collision(int64_t m) const {
    return cfg.mpc_every - (int)(m % cfg.mpc_every);
  }

  int do_rebuild(int64_t n, int tc, bool mpc, bool free_flight = false) {
    StepArgs a = args(n);
    a.tc = tc;
    a.tc_full = (int)(n - last_full);
    a.mpc = mpc ? 1 : 0;
    const bool collision_step = n % cfg.mpc_every == 0;
    // free-flight shell members and deferred far particles only between collision steps
    a.horizon = (free_flight && !collision_step) ? steps_to_collision(n) : 0;
    a.full = (!free_flight || collision_step) ? 1 : 0;
    bool sort_now = cfg.sort_every > 0 && n % cfg.sort_every == 0;
    const bool resort_now = !sort_now && mpc && collision_step && resort_every > 0 && n % resort_every == 0;
    if (a.full || sort_now) watch_valid = false;
    a.use_watch = watch_valid ? 1 : 0;
    pb(PROF_BINS); Launch<T>::build_bins(d, kp, a.full ? 0 : a.tc_full, st); pe();
    if (resort_now) { pb(PROF_SORT); resort(a.tc, a.tc_full); pe(); }
    if (sort_now) {
      StepArgs m = a;
      m.merge_only = 1;
      m.mpc = 0;
      m.full = 1;
      pb(PROF_REBUILD); Launch<T>::rebuild(d, kp, m, st); pe();
      pb(PROF_SORT); Launch<T>::sort(d, kp, st); pe();
      a.tc = 0;
      a.tc_full = 0;
      a.full = 1;
    }
    // a collision step's full pass runs split: far particles in a lean pass,
    // the rest through the list kernel
    if (a.full && a.mpc) { pb(PROF_REBUILD); Launch<T>::rebuild_split(d, kp, a, st); pe(); }
    else { pb(PROF_REBUILD); Launch<T>::rebuild(d, kp, a, st); pe(); }
    pb(PROF_FINALIZE); Launch<T>::finalize_rebuild(d, kp, a, cfg.skin, st); pe();
    // a collision step's shell is used once before it is sorted into free-flight
    // and active members; other rebuilds order theirs for the coming steps
    const bool sorted = (!collision_step || !free_flight) && kp.ns > 0;
    if (sorted) { pb(PROF_FINALIZE); Launch<T>::sort_shell(d, kp, st); pe(); }
    Counters h;
    int r = read_counters(h);
    if (r) return r;
    if (h.abort_step) return -1;
    if (h.status) return dev_status_to_api(h.status);
    if (!sorted) std::swap(d.sh, d.sh2);   // (sort_shell filled d.sh)
    n_inside = h.n_inside;
    time_penetrate = h.time_penetrate;
    time_count = 0;
    last_rebuild = n;
    if (a.full) last_full = n;
    home_shell = true;
    prepared = true;
    return MPCMD_OK;
  }

  int prepare() override {
    // main_pattern.f95:168-187 (the reactive grid table is built at create)
    if (advanced) return MPCMD_ERR_STATE;
    if (prepared) {
      // a context that has stepped since its state was set: a full list pass
      // streams the lazily moved outside particles to this step and the flush
      // writes the shell members back, so the run restarts from the state of
      // this step
      regather_shell();
      int r = do_rebuild(cstep, time_count, false);
      if (r) return r < 0 ? MPCMD_ERR_STATE : r;
      flush_shell();
    }
    home_shell = false;
    watch_valid = false;
    advanced = false;
    CK(cudaMemsetAsync(d.ctr, 0, sizeof(Counters), st));
    if (kp.ns > 0) Launch<T>::update_srel(d, kp, st);
    if (cfg.sort_every > 0 && cstep % cfg.sort_every == 0) {
      Launch<T>::sort(d, kp, st);
    }
    Launch<T>::build_bins(d, kp, 0, st);
    StepArgs a = args(cstep);
    a.full = 1;
    Launch<T>::rebuild(d, kp, a, st);
    Launch<T>::finalize_rebuild(d, kp, a, cfg.skin, st);
    Launch<T>::sort_shell(d, kp, st);
    Counters h;
    int r = read_counters(h);
    if (r) return r;
    if (h.status) return dev_status_to_api(h.status);
    if (kp.ns == 0) std::swap(d.sh, d.sh2);   // (with spheres sort_shell filled d.sh)
    // the first half kick of the run uses zero pair forces, as after
    // initial_mod.f95 (FpairX = 0), or after a restart the forces of the
    // state (restart_mod.f95:415-528: pair forces, catalysis, sphere totals;
    // no kick)
    CK(cudaMemsetAsync(d.sh.pf, 0, sizeof(T) * 3 * PAIRMAX * (size_t)d.sh.cap, st));
    if (restart_pending) {
      StepArgs f = args(cstep);
      f.forces_only = 1;
      f.rebuilt = 1;
      Launch<T>::force(d, kp, f, st);
      Launch<T>::sphere_totals(d, kp, w3, st);
      Counters hf;
      if ((r = read_counters(hf))) return r;
      if (hf.status) return dev_status_to_api(hf.status);
      restart_pending = false;
    }
    CK(cudaStreamSynchronize(st));
    n_inside = h.n_inside;
    time_penetrate = h.time_penetrate;
    time_count = 0;
    last_rebuild = cstep;
    last_full = cstep;
    home_shell = true;
    prepared = true;
    return MPCMD_OK;
  }

  int prepare_restart() override {
    restart_pending = true;
    return prepare();
  }

  int handle_abort(int step) {
    // the displacement criterion of evolve_mod.f95:465 fired at `step`: every
    // kernel from that step's force evaluation on was skipped
    cstep = step - 1;
    time_count = (int)(cstep - last_rebuild);
    advanced = true;
    force_rebuild_step = step;
    CK(cudaMemsetAsync(&d.ctr->abort_step, 0, sizeof(int), st));
    return MPCMD_OK;
  }

  // nsteps iterations of the main loop (main_pattern.f95:203-225); with_mpc
  // false runs evolve only (the collision stages are separate calls).
  int run(int64_t nsteps, bool with_mpc) override {
    if (!prepared) return MPCMD_ERR_STATE;
    if (nsteps <= 0) return MPCMD_OK;
    regather_shell();
    const int64_t target = cstep + nsteps;
    while (cstep < target) {
      const int64_t n = cstep + 1;
      const bool last = (n == target);
      if (!advanced) {
        StepArgs a = args(n - 1);
        a.advance = 1;
        // right after a rebuild the shell can be sorted into free-flight and active members
        a.horizon = time_count == 0 ? steps_to_collision(n - 1) : 0;
        pb(PROF_SHELL_ADVANCE); Launch<T>::advance(d, kp, a, st); pe();
        if (a.horizon > 0) {   // the packed shell in d.sh2 is sorted back into d.sh
          Launch<T>::sort_shell(d, kp, st);
          if (kp.ns == 0) std::swap(d.sh, d.sh2);
        }
        pb(PROF_DIMER); Launch<T>::dimer(d, kp, a, 2, w3, cfg.rattle_max_iter, st); pe();
        advanced = true;
      }
      time_count += 1;
      const bool mpc_step = (n % cfg.mpc_every) == 0;
      const bool mpc = mpc_step && with_mpc;
      const bool rebuild = mpc_step || time_count == time_penetrate || force_rebuild_step == n;
      if (mpc) draw_shift(n);
      if (rebuild) {
        force_rebuild_step = -1;
        int r = do_rebuild(n, time_count, mpc, true);
        if (r == -1) {
          Counters h;
          if ((r = read_counters(h))) return r;
          handle_abort(h.abort_step);
          continue;
        }
        if (r) return r;
      }
      StepArgs a = args(n);
      a.tc = time_count;
      a.mpc = mpc ? 1 : 0;
      a.rebuilt = rebuild ? 1 : 0;
      a.advance = last ? 0 : 1;
      pb(PROF_FORCE); Launch<T>::force(d, kp, a, st); pe();
      if (mpc && kp.kinetics == MPCMD_KIN_SELKOV && kp.exclusion == MPCMD_EXCL_CELLS) {
        pb(PROF_AFFECTED); Launch<T>::affected(d, kp, a, st); pe();
      }
      pb(PROF_DIMER); Launch<T>::dimer(d, kp, a, 1 | (last ? 0 : 2), w3, cfg.rattle_max_iter, st); pe();
      if (mpc) {
        pb(PROF_CELLS); Launch<T>::cells(d, kp, a, 1 | (kp.kinetics ? 2 : 0), st); pe();
        // the rotated velocities hold until the next collision: the particles
        // that can come near a sphere or a wall before it form the watch list
        CK(cudaMemsetAsync(&d.ctr->n_watch, 0, sizeof(unsigned int), st));
        CK(cudaMemsetAsync(&d.ctr->vfar, 0, sizeof(unsigned long long), st));
        pb(PROF_BINS); Launch<T>::gap_field(d, kp, cfg.mpc_every, st); pe();
        a.watch_build = cfg.mpc_every;
        pb(PROF_ROTATE_MAIN); Launch<T>::rotate_main(d, kp, a, st); pe();
        StepArgs ar = a;
        ar.horizon = a.advance ? cfg.mpc_every : 0;   // the rebuild of this step was the last one
        pb(PROF_SHELL_ADVANCE); Launch<T>::rotate_shell(d, kp, ar, st); pe();
        if (ar.horizon > 0) {
          pb(PROF_SHELL_ADVANCE); Launch<T>::sort_shell(d, kp, st); pe();
          if (kp.ns == 0) std::swap(d.sh, d.sh2);
        }
        watch_valid = true;
      }
      advanced = !last;
      cstep = n;
      if (last) {
        Counters h;
        int r = read_counters(h);
        if (r) return r;
        if (h.abort_step) { handle_abort(h.abort_step); continue; }
        if (h.status) return dev_status_to_api(h.status);
      }
    }
    return MPCMD_OK;
  }

  // ---------------------------------------------------------- stages ----
  int sort_stage() override {
    if (advanced) return MPCMD_ERR_STATE;
    flush_shell();
    Launch<T>::sort(d, kp, st);
    prepared = false;
    CK(cudaMemsetAsync(&d.ctr->n_inside, 0, sizeof(unsigned int), st));
    n_inside = 0;
    CK(cudaStreamSynchronize(st));
    return MPCMD_OK;
  }

  int rebuild_stage() override {
    if (advanced) return MPCMD_ERR_STATE;
    int r = do_rebuild(cstep, time_count, false);
    return r < 0 ? MPCMD_ERR_STATE : r;
  }

  int distribute_stage() override {
    if (advanced) return MPCMD_ERR_STATE;
    flush_shell();
    if (kp.ns > 0) Launch<T>::build_bins(d, kp, 0, st);
    CK(cudaMemsetAsync(d.dcnt, 0, 4 * (size_t)kp.ncell, st));
    CK(cudaMemsetAsync(d.dfirst, 0xFF, 16 * (size_t)kp.ncell, st));
    CK(cudaMemsetAsync(d.affected, 0, (size_t)kp.ncell, st));
    StepArgs a = args(cstep);
    Launch<T>::accumulate_main(d, kp, a, 2, st);
    if (kp.exclusion == MPCMD_EXCL_CELLS) Launch<T>::affected(d, kp, a, st);
    CK(cudaStreamSynchronize(st));
    return check_device_status();
  }

  int rotation_stage() override {
    if (advanced) return MPCMD_ERR_STATE;
    flush_shell();
    draw_shift(cstep);
    StepArgs a = args(cstep);
    Launch<T>::accumulate_main(d, kp, a, 1, st);
    snapshot_counts();
    Launch<T>::cells(d, kp, a, 1, st);
    Launch<T>::rotate_main(d, kp, a, st);
    CK(cudaStreamSynchronize(st));
    return check_device_status();
  }

  std::vector<int32_t> counts_snapshot;
  void snapshot_counts() {
    counts_snapshot.assign((size_t)kp.ncell_shift, 0);
    if (sizeof(T) == 4) {
      std::vector<float> a((size_t)kp.ncell_shift * 4);
      cudaMemcpyAsync(a.data(), d.acc, a.size() * 4, cudaMemcpyDeviceToHost, st);
      cudaStreamSynchronize(st);
      for (int64_t c = 0; c < kp.ncell_shift; ++c) counts_snapshot[(size_t)c] = (int32_t)a[(size_t)(4 * c)];
    } else {
      std::vector<double> a((size_t)kp.ncell_shift * 4);
      cudaMemcpyAsync(a.data(), d.acc, a.size() * 8, cudaMemcpyDeviceToHost, st);
      cudaStreamSynchronize(st);
      for (int64_t c = 0; c < kp.ncell_shift; ++c) counts_snapshot[(size_t)c] = (int32_t)a[(size_t)(4 * c)];
    }
  }

  int reaction_stage() override {
    if (advanced) return MPCMD_ERR_STATE;
    flush_shell();
    StepArgs a = args(cstep);
    Launch<T>::cells(d, kp, a, 2, st);
    CK(cudaStreamSynchronize(st));
    return check_device_status();
  }

  // ----------------------------------------------------------- initial ----
  int initial() override {
    // initial_mod.f95:78-119: dimers by rejection with contract draws
    const double cut = std::pow(2.0, 1.0 / 6.0);
    const double rc = cfg.rc, rn = cfg.rn, dcn = cfg.dcn;
    const double wcC = (cfg.rw + rc) * w3, wcN = (cfg.rw + rn) * w3;
    const bool per = cfg.geometry == MPCMD_GEOM_PERIODIC;
    const double L[3] = {(double)cfg.lx, (double)cfg.ly, (double)cfg.lz};
    std::vector<double> pos(3 * (size_t)kp.ns, 0.0);
    auto wrapf = [](double x, double Lq) { return x - Lq * std::floor(x / Lq); };
    auto mi = [](double dd, double Lq) {
      if (dd > 0.5 * Lq) dd -= Lq;
      else if (dd < -0.5 * Lq) dd += Lq;
      return dd;
    };
    if (cfg.layout != MPCMD_LAYOUT_RANDOM) {
      // rotational_code/2d_array/initial_mod.f95:68-90 (grid, row-major over
      // numrows x numcols) and linear_periodic_ci/initial_mod.f95:72-88 (line
      // along x): motor centres at the pitch Dcn + 2 Rc 2^(1/6) + sep in the
      // plane z = zdimeq, each with a uniform in-plane orientation
      const bool grid = cfg.layout == MPCMD_LAYOUT_GRID;
      const double sep = cfg.layout_sep, rows = cfg.layout_rows, cols = cfg.layout_cols;
      for (int i = 0; i < cfg.n_dimers; ++i) {
        double theta, unused;
        contract_pair(cfg.seed, TAG_INIT_DIMER, (uint32_t)i, 0, 0, theta, unused);
        theta = 2. * kPi * theta;
        const double w = dcn + 2. * rc * cut;
        double cx, cy;
        if (grid) {
          const int64_t j = i / cfg.layout_cols + 1, k = i % cfg.layout_cols + 1;
          cx = 0.5 * (L[0] - w * cols - sep * (cols - 1)) + 0.5 * w + (double)(k - 1) * (w + sep);
          cy = 0.5 * (L[1] - (w + sep) * (rows - 1) - w) + 0.5 * w + (double)(j - 1) * (w + sep);
        } else {
          cx = 0.5 * sep + 0.5 * w + (double)i * (w + sep);
          cy = L[1] * 0.5;
        }
        double* X1 = &pos[3 * (2 * i)];
        double* X2 = &pos[3 * (2 * i + 1)];
        X1[0] = cx + 0.5 * dcn * std::cos(theta); X1[1] = cy + 0.5 * dcn * std::sin(theta); X1[2] = cfg.tether_z;
        X2[0] = cx - 0.5 * dcn * std::cos(theta); X2[1] = cy - 0.5 * dcn * std::sin(theta); X2[2] = cfg.tether_z;
      }
    }
    for (int i = 0; i < cfg.n_dimers && cfg.layout == MPCMD_LAYOUT_RANDOM; ++i) {
      int64_t at;
      for (at = 0; at < 100000000; ++at) {
        double ux, uy, uz, uphi, uth, unused;
        contract_pair(cfg.seed, TAG_INIT_DIMER, (uint32_t)i, (uint32_t)at, 0, ux, uy);
        contract_pair(cfg.seed, TAG_INIT_DIMER, (uint32_t)i, (uint32_t)at, 1, uz, uphi);
        contract_pair(cfg.seed, TAG_INIT_DIMER, (uint32_t)i, (uint32_t)at, 2, uth, unused);
        double phi = 2.0 * kPi * uphi, theta = 2.0 * uth - 1.0;
        if (cfg.init_plane) { uz = 0.5; theta = 0.0; }
        double s = std::sqrt(1.0 - theta * theta);
        double P[2][3] = {{L[0] * ux + 0.5 * dcn * (s * std::cos(phi)), L[1] * uy + 0.5 * dcn * (s * std::sin(phi)),
                           L[2] * uz + 0.5 * dcn * theta},
                          {L[0] * ux - 0.5 * dcn * (s * std::cos(phi)), L[1] * uy - 0.5 * dcn * (s * std::sin(phi)),
                           L[2] * uz - 0.5 * dcn * theta}};
        for (int u = 0; u < 2; ++u) {
          P[u][0] = wrapf(P[u][0], L[0]);
          P[u][1] = wrapf(P[u][1], L[1]);
          if (per) P[u][2] = wrapf(P[u][2], L[2]);
        }
        bool bad = false;
        if (!per && !cfg.init_plane)
          bad = P[0][2] < wcC + rc * cut || P[0][2] > L[2] - wcC - rc * cut || P[1][2] < wcN + rn * cut ||
                P[1][2] > L[2] - wcN - rn * cut;
        for (int j = 0; j < i && !bad; ++j)
          for (int u = 0; u < 2 && !bad; ++u)
            for (int v = 0; v < 2 && !bad; ++v) {
              double dd[3];
              for (int q = 0; q < 3; ++q) dd[q] = P[u][q] - pos[3 * (2 * j + v) + q];
              // minimum image in the periodic directions (x, y always; z when periodic)
              for (int q = 0; q < (per ? 3 : 2); ++q) dd[q] = mi(dd[q], L[q]);
              double r = (u == 0 ? rc : rn) + (v == 0 ? rc : rn);
              double lim = (r * cut) * (r * cut);
              if (u == 0 && v == 0) lim = (2. * rc * cut) * (2. * rc * cut);
              if (u == 1 && v == 1) lim = (2. * rn * cut) * (2. * rn * cut);
              if (dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2] < lim) bad = true;
            }
        if (!bad) {
          for (int q = 0; q < 3; ++q) { pos[3 * (2 * i) + q] = P[0][q]; pos[3 * (2 * i + 1) + q] = P[1][q]; }
          break;
        }
      }
      if (at == 100000000) return MPCMD_ERR_INIT;
    }
    int64_t acc = 0, bounds[4];
    for (int c = 0; c < 4; ++c) { acc += cfg.init_count[c]; bounds[c] = acc; }
    if (acc != kp.n) return MPCMD_ERR_CONFIG;
    const size_t nb = sizeof(double) * 3 * (size_t)kp.ns;
    if (kp.ns > 0) {
      CK(cudaMemcpyAsync(d.dpos, pos.data(), nb, cudaMemcpyHostToDevice, st));
      CK(cudaMemsetAsync(d.dvel, 0, nb, st));
      CK(cudaMemsetAsync(d.dfrc, 0, nb, st));
      Launch<T>::update_srel(d, kp, st);
      int r = set_anchors(midpoints(pos.data()).data());
      if (r) return r;
    }
    CK(cudaMemsetAsync(d.ctr, 0, sizeof(Counters), st));
    Launch<T>::build_bins(d, kp, 0, st);
    Launch<T>::init_solvent(d, kp, bounds, cfg.kT, cfg.mass, st);
    d.lid = d.lpos = nullptr;
    if (d.owner) CK(cudaMemsetAsync(d.owner, 0, sizeof(uint16_t) * (size_t)kp.n, st));
    if (d.inc) CK(cudaMemsetAsync(d.inc, 0, (size_t)kp.n, st));
    CK(cudaStreamSynchronize(st));
    prepared = false; home_shell = false; advanced = false; n_inside = 0;
    restart_pending = false;
    cstep = 0; time_count = 0;
    Counters h;
    int r = read_counters(h);
    if (r) return r;
    CK(cudaMemsetAsync(d.ctr, 0, sizeof(Counters), st));
    CK(cudaStreamSynchronize(st));
    return dev_status_to_api(h.status);
  }

  // -------------------------------------------------------- inspection ----
  int observables(mpcmd_obs* o) override {
    std::memset(o, 0, sizeof(*o));
    CK(cudaMemsetAsync(d.ctr->sums, 0, 8 * sizeof(double), st));
    Launch<T>::observables(d, kp, cfg.mass, grid, st);
    Counters h;
    int r = read_counters(h);
    if (r) return r;
    std::vector<double> dv(3 * (size_t)kp.ns), dp((size_t)std::max(kp.nd, 1));
    if (kp.ns > 0) {
      CK(cudaMemcpy(dv.data(), d.dvel, dv.size() * 8, cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(dp.data(), d.dpot, (size_t)kp.nd * 8, cudaMemcpyDeviceToHost));
    }
    double pd[3] = {0, 0, 0}, ked = 0, pot = 0;
    for (int s = 0; s < kp.ns; ++s) {
      double m = (s % 2 == 0) ? cfg.mc : cfg.mn;
      for (int c = 0; c < 3; ++c) { pd[c] += m * dv[3 * s + c]; ked += 0.5 * m * dv[3 * s + c] * dv[3 * s + c]; }
    }
    for (int k = 0; k < kp.nd; ++k) pot += dp[(size_t)k];
    for (int c = 0; c < 3; ++c) { o->solvent_momentum[c] = h.sums[c]; o->momentum[c] = h.sums[c] + pd[c]; }
    o->kinetic_solvent = h.sums[3];
    o->kinetic_dimer = ked;
    o->potential = pot;
    for (int c = 0; c < 4; ++c) o->species_count[c] = (int64_t)llround(h.sums[4 + c]);
    o->n_inside = h.n_inside;
    o->time_count = time_count;
    o->time_penetrate = time_penetrate;
    o->cstep = cstep;
    return dev_status_to_api(h.status);
  }

  // output_mod.f95:482-575 on the device: a flush of the shell, one counting
  // pass over the particles, normalisation on the host.  Allocates its count
  // arrays per call (an output-cadence call, not part of the step).
  int concentration(const mpcmd_conc_params* p, double* totals, double* const* fields) override {
    if (!(p->x_width > 0 && p->y_width > 0 && p->z_width > 0 && p->half_width >= 0)) return MPCMD_ERR_CONFIG;
    const double L[3] = {(double)cfg.lx, (double)cfg.ly, (double)cfg.lz};
    const int64_t nx = (int64_t)(L[0] / p->x_width), ny = (int64_t)(L[1] / p->y_width), nz = (int64_t)(L[2] / p->z_width);
    if (nx < 1 || ny < 1 || nz < 1 || nx > (1 << 20) || ny > (1 << 20) || nz > (1 << 20)) return MPCMD_ERR_CONFIG;
    if (nx * ny > (int64_t)1 << 28 || nx * nz > (int64_t)1 << 28 || ny * nz > (int64_t)1 << 28) return MPCMD_ERR_CONFIG;
    if (advanced) return MPCMD_ERR_STATE;
    flush_shell();
    const int64_t sz[8] = {nx, nx, nx * ny, nx * ny, nx * nz, nx * nz, ny * nz, ny * nz};
    int64_t off[9];
    off[0] = 0;
    for (int q = 0; q < 8; ++q) off[q + 1] = off[q] + sz[q];
    uint32_t* cnt = nullptr;
    unsigned long long* tot = nullptr;
    if (cudaMalloc(&cnt, sizeof(uint32_t) * (size_t)off[8]) != cudaSuccess) return MPCMD_ERR_CUDA;
    if (cudaMalloc(&tot, 2 * sizeof(unsigned long long)) != cudaSuccess) { cudaFree(cnt); return MPCMD_ERR_CUDA; }
    int r = MPCMD_OK;
    std::vector<uint32_t> h((size_t)off[8]);
    unsigned long long ht[2] = {0, 0};
    ConcArgs c;
    c.xs = p->x_slab; c.ys = p->y_slab; c.zs = p->z_slab; c.hw = p->half_width;
    c.xw = p->x_width; c.yw = p->y_width; c.zw = p->z_width;
    c.nx = (int)nx; c.ny = (int)ny; c.nz = (int)nz;
    uint32_t* ptrs[8];
    for (int q = 0; q < 8; ++q) ptrs[q] = cnt + off[q];
    c.c1a = ptrs[0]; c.c1b = ptrs[1]; c.xya = ptrs[2]; c.xyb = ptrs[3];
    c.xza = ptrs[4]; c.xzb = ptrs[5]; c.yza = ptrs[6]; c.yzb = ptrs[7];
    c.tot = tot;
    if (cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * (size_t)off[8], st) != cudaSuccess ||
        cudaMemsetAsync(tot, 0, 2 * sizeof(unsigned long long), st) != cudaSuccess) {
      r = MPCMD_ERR_CUDA;
    } else {
      Launch<T>::concentration(d, kp, time_count, (int)(last_rebuild - last_full), c, st);
      if (cudaMemcpyAsync(h.data(), cnt, sizeof(uint32_t) * h.size(), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaMemcpyAsync(ht, tot, sizeof(ht), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        r = MPCMD_ERR_CUDA;
    }
    cudaFree(cnt);
    cudaFree(tot);
    if (r) return r;
    const double hw2 = 2.0 * p->half_width;
    const double vol = (double)(int64_t)(L[0] * L[1] * L[2]);
    const double v[8] = {p->x_width * L[1] * hw2, p->x_width * L[1] * hw2,
                         p->x_width * p->y_width * hw2, p->x_width * p->y_width * hw2,
                         p->x_width * p->z_width * hw2, p->x_width * p->z_width * hw2,
                         p->y_width * p->z_width * hw2, p->y_width * p->z_width * hw2};
    if (totals) {
      totals[0] = (double)ht[0]; totals[1] = (double)ht[1];
      totals[2] = (double)ht[0] / vol; totals[3] = (double)ht[1] / vol;
    }
    for (int q = 0; q < 8; ++q) {
      if (!fields[q]) continue;
      for (int64_t j = 0; j < sz[q]; ++j) fields[q][j] = (double)h[(size_t)(off[q] + j)] / v[q];
    }
    return check_device_status();
  }

  // Dimer axes from the FP64 sphere state: output_mod.f95:826-846 (d / Dcn)
  // or Output_SelkovDimer.f90:146-172 (unit vector, propulsion speed).
  int dimer_axes(int normalize, double* nucvec, double* vdot) override {
    if (normalize != 0 && normalize != 1) return MPCMD_ERR_CONFIG;
    if (kp.nd == 0) return MPCMD_OK;
    std::vector<double> X(3 * (size_t)kp.ns), V(3 * (size_t)kp.ns);
    CK(cudaMemcpyAsync(X.data(), d.dpos, X.size() * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(V.data(), d.dvel, V.size() * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const double L[3] = {(double)cfg.lx, (double)cfg.ly, (double)cfg.lz};
    const bool per[3] = {true, true, cfg.geometry == MPCMD_GEOM_PERIODIC};
    for (int k = 0; k < kp.nd; ++k) {
      double dd[3];
      for (int c = 0; c < 3; ++c) {
        dd[c] = X[6 * (size_t)k + c] - X[6 * (size_t)k + 3 + c];
        if (per[c]) {
          if (dd[c] > 0.5 * L[c]) dd[c] -= L[c];
          else if (dd[c] < -0.5 * L[c]) dd[c] += L[c];
        }
      }
      const double len = std::sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
      const double den = normalize ? len : cfg.dcn;
      if (nucvec)
        for (int c = 0; c < 3; ++c) nucvec[3 * (size_t)k + c] = dd[c] / den;
      if (vdot) {
        double s = 0.0;
        for (int c = 0; c < 3; ++c) {
          const double vcm = (cfg.mc * V[6 * (size_t)k + c] + cfg.mn * V[6 * (size_t)k + 3 + c]) / (cfg.mn + cfg.mc);
          s += vcm * (dd[c] / len);
        }
        vdot[k] = s;
      }
    }
    return MPCMD_OK;
  }

  int get_new_cell(int64_t* out) override {
    std::vector<uint32_t> lid;
    int r = host_lid(lid);
    if (r) return r;
    std::vector<uint32_t> k((size_t)kp.n);
    CK(cudaMemcpy(k.data(), d.skey, k.size() * 4, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < k.size(); ++i) out[lid.empty() ? i : lid[i]] = k[i];
    return MPCMD_OK;
  }

  int get_cell_rotation(double* cm, double* axis, int32_t* count) override {
    std::vector<T> r((size_t)kp.ncell_shift * 6);
    CK(cudaMemcpy(r.data(), d.rot, r.size() * sizeof(T), cudaMemcpyDeviceToHost));
    for (int64_t c = 0; c < kp.ncell_shift; ++c)
      for (int q = 0; q < 3; ++q) {
        if (cm) cm[3 * c + q] = (double)r[(size_t)(6 * c + q)];
        if (axis) axis[3 * c + q] = (double)r[(size_t)(6 * c + 3 + q)];
      }
    if (count)
      for (int64_t c = 0; c < kp.ncell_shift; ++c)
        count[c] = (size_t)c < counts_snapshot.size() ? counts_snapshot[(size_t)c] : 0;
    return MPCMD_OK;
  }

  int get_distribute(int32_t* counts, int64_t* first) override {
    std::vector<uint32_t> cn((size_t)kp.ncell);
    std::vector<uint32_t> fk((size_t)kp.ncell * 4);
    CK(cudaMemcpy(cn.data(), d.dcnt, cn.size() * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(fk.data(), d.dfirst, fk.size() * 4, cudaMemcpyDeviceToHost));
    for (int64_t c = 0; c < kp.ncell; ++c)
      for (int s = 0; s < 4; ++s) {
        if (counts) counts[4 * c + s] = (int32_t)((cn[(size_t)c] >> (8 * s)) & 255u);
        const uint32_t key = fk[(size_t)(4 * c + s)];
        if (first) first[4 * c + s] = key == 0xFFFFFFFFu ? -1 : (int64_t)(key & 0x7FFFFFFFu);
      }
    return MPCMD_OK;
  }

  int get_affected(int32_t* a) override {
    std::vector<uint8_t> v((size_t)kp.ncell);
    CK(cudaMemcpy(v.data(), d.affected, v.size(), cudaMemcpyDeviceToHost));
    for (size_t c = 0; c < v.size(); ++c) a[c] = v[c];
    return MPCMD_OK;
  }

  int get_inside(int64_t* n, int64_t* idx) override {
    Counters h;
    int r = read_counters(h);
    if (r) return r;
    std::vector<uint32_t> lid;
    r = host_lid(lid);
    if (r) return r;
    auto main_index = [&](size_t i) -> int64_t { return lid.empty() ? (int64_t)i : (int64_t)lid[i]; };
    // the shell buffer, then the free-flight members kept in the main home
    std::vector<uint8_t> fl((size_t)kp.n);
    CK(cudaMemcpy(fl.data(), d.p.flag, fl.size(), cudaMemcpyDeviceToHost));
    int64_t m = h.n_inside;
    for (size_t i = 0; i < fl.size(); ++i) m += (fl[i] & FLAG_PASSIVE) ? 1 : 0;
    *n = m;
    if (idx) {
      std::vector<uint32_t> v(h.n_inside);
      if (h.n_inside) CK(cudaMemcpy(v.data(), d.sh.idx, v.size() * 4, cudaMemcpyDeviceToHost));
      size_t k = 0;
      for (; k < v.size(); ++k) idx[k] = main_index(v[k]);
      for (size_t i = 0; i < fl.size(); ++i)
        if (fl[i] & FLAG_PASSIVE) idx[k++] = main_index(i);
    }
    return MPCMD_OK;
  }

  int get_pairs(int64_t* np, int64_t* part, int32_t* sph) override {
    Counters h;
    int r = read_counters(h);
    if (r) return r;
    std::vector<uint32_t> lid;
    r = host_lid(lid);
    if (r) return r;
    size_t m = h.n_inside;
    std::vector<uint32_t> idx(m);
    std::vector<uint8_t> cnt(m);
    std::vector<uint16_t> sp(m * PAIRMAX);
    if (m) {
      CK(cudaMemcpy(idx.data(), d.sh.idx, m * 4, cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(cnt.data(), d.sh.np, m, cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(sp.data(), d.sh.sph, m * PAIRMAX * 2, cudaMemcpyDeviceToHost));
    }
    int64_t k = 0;
    for (size_t j = 0; j < m; ++j)
      for (int q = 0; q < cnt[j]; ++q) {
        if (part) part[k] = lid.empty() ? (int64_t)idx[j] : (int64_t)lid[idx[j]];
        if (sph) sph[k] = sp[j * PAIRMAX + q];
        ++k;
      }
    *np = k;
    return MPCMD_OK;
  }

  int get_counters(int64_t* c, int32_t n) override {
    Counters h;
    int r = read_counters(h);
    if (r) return r;
    int64_t v[15] = {(int64_t)h.n_inside, (int64_t)h.status, (int64_t)h.time_penetrate, (int64_t)h.rattle_iters,
                     (int64_t)cstep, (int64_t)time_count, (int64_t)h.abort_step, (int64_t)last_rebuild,
                     (int64_t)h.dbg_code, (int64_t)h.dbg_val, (int64_t)h.n_watch, (int64_t)h.acc_force,
                     (int64_t)h.acc_rebuild, (int64_t)h.acc_placed, resorts};
    for (int q = 0; q < n && q < 15; ++q) c[q] = v[q];
    return MPCMD_OK;
  }

  int checkpoint(const char* path) override;
  int restore(const char* path) override;

  int event_record(int slot) override {
    if (slot < 0 || slot >= 8) return MPCMD_ERR_CONFIG;
    if (!marks[slot]) CK(cudaEventCreate(&marks[slot]));
    CK(cudaEventRecord(marks[slot], st));
    return MPCMD_OK;
  }
  int event_elapsed(int a, int b, double* ms) override {
    if (a < 0 || a >= 8 || b < 0 || b >= 8 || !marks[a] || !marks[b]) return MPCMD_ERR_STATE;
    CK(cudaEventSynchronize(marks[b]));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, marks[a], marks[b]));
    *ms = f;
    return MPCMD_OK;
  }
  int synchronize() override {
    CK(cudaStreamSynchronize(st));
    return MPCMD_OK;
  }
  int profile(int enable) override {
    prof_collect();
    profiling = enable != 0;
    if (enable) {
      for (int k = 0; k < PROF_KINDS; ++k) { prof_ms[k] = 0.; prof_n[k] = 0; }
      CK(cudaMemsetAsync(&d.ctr->acc_force, 0, 3 * sizeof(unsigned long long), st));
    }
    return MPCMD_OK;
  }
  int profile_read(double* ms, int64_t* count, int n) override {
    prof_collect();
    for (int k = 0; k < n && k < PROF_KINDS; ++k) { ms[k] = prof_ms[k]; count[k] = prof_n[k]; }
    return MPCMD_OK;
  }
};

// ------------------------------------------------------- checkpoint ----
// Device-state snapshot (the role of restart_mod.f95 / Restart.f90 plus the
// RNG position, which for counter-based streams is the step counter).  The
// file is written to <path>.tmp and renamed, so an interrupted write keeps the
// previous checkpoint; a checksum guards the payload.  Version 2 files hold
// every particle at the checkpoint step (the outside particles streamed over
// their pending lag, time_count 0) and the rotor anchors, so a restored and
// prepared context goes on as the original one does after mpcmd_prepare;
// version 1 files (the reference's view, the lag in time_count) still load.
struct CkptHeader {
  char magic[8];
  int32_t version, precision;
  int64_t n, ns, cstep;
  int32_t time_count, lx, ly, lz;
  uint64_t seed;
  uint64_t checksum;
};

uint64_t fnv1a(const void* p, size_t n, uint64_t h) {
  const unsigned char* b = (const unsigned char*)p;
  for (size_t i = 0; i < n; ++i) { h ^= b[i]; h *= 1099511628211ull; }
  return h;
}

template <typename T>
int Engine<T>::checkpoint(const char* path) {
  if (advanced) return MPCMD_ERR_STATE;
  const int64_t n = kp.n, ns = kp.ns;
  std::vector<double> buf((size_t)(6 * n + 9 * ns));
  std::vector<int32_t> fl((size_t)n);
  // version 2: every particle at the current step (time_count 0 on restore)
  int r = download_state(buf.data(), buf.data() + n, buf.data() + 2 * n, buf.data() + 3 * n, buf.data() + 4 * n,
                         buf.data() + 5 * n, fl.data(), buf.data() + 6 * n, buf.data() + 6 * n + 3 * ns,
                         buf.data() + 6 * n + 6 * ns, true);
  if (r) return r;
  std::vector<double> anc(3 * (size_t)kp.nd);
  r = get_anchors(anc.data());
  if (r) return r;
  std::vector<int32_t> tags(d.owner ? (size_t)n : 0);
  if (d.owner && (r = get_owner_tags(tags.data()))) return r;
  CkptHeader h{};
  std::memcpy(h.magic, "MPCMDCK1", 8);
  h.version = 2; h.precision = (int32_t)(sizeof(T) * 8);
  h.n = n; h.ns = ns; h.cstep = cstep; h.time_count = 0;
  h.lx = kp.lx; h.ly = kp.ly; h.lz = kp.lz; h.seed = cfg.seed;
  uint64_t cs = fnv1a(buf.data(), buf.size() * 8, 1469598103934665603ull);
  cs = fnv1a(fl.data(), fl.size() * 4, cs);
  cs = fnv1a(anc.data(), anc.size() * 8, cs);
  h.checksum = fnv1a(tags.data(), tags.size() * 4, cs);
  std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return MPCMD_ERR_IO;
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 && std::fwrite(buf.data(), 8, buf.size(), f) == buf.size() &&
            std::fwrite(fl.data(), 4, fl.size(), f) == fl.size() &&
            std::fwrite(anc.data(), 8, anc.size(), f) == anc.size() &&
            std::fwrite(tags.data(), 4, tags.size(), f) == tags.size();
  ok = (std::fclose(f) == 0) && ok;
  if (!ok || std::rename(tmp.c_str(), path) != 0) { std::remove(tmp.c_str()); return MPCMD_ERR_IO; }
  return MPCMD_OK;
}

template <typename T>
int Engine<T>::restore(const char* path) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return MPCMD_ERR_IO;
  CkptHeader h{};
  if (std::fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, "MPCMDCK1", 8) != 0 || h.n != kp.n ||
      h.ns != kp.ns || h.lx != kp.lx || h.ly != kp.ly || h.lz != kp.lz || h.version < 1 || h.version > 2) {
    std::fclose(f);
    return MPCMD_ERR_CHECKPOINT;
  }
  const int64_t n = kp.n, ns = kp.ns;
  std::vector<double> buf((size_t)(6 * n + 9 * ns));
  std::vector<int32_t> fl((size_t)n);
  // version 1 files end with the flags; version 2 adds the rotor anchors
  std::vector<double> anc(h.version >= 2 ? 3 * (size_t)kp.nd : 0);
  std::vector<int32_t> tags(h.version >= 2 && d.owner ? (size_t)n : 0);
  bool ok = std::fread(buf.data(), 8, buf.size(), f) == buf.size() && std::fread(fl.data(), 4, fl.size(), f) == fl.size() &&
            std::fread(anc.data(), 8, anc.size(), f) == anc.size() &&
            std::fread(tags.data(), 4, tags.size(), f) == tags.size();
  ok = ok && std::fgetc(f) == EOF;   // nothing left: the file matches this configuration
  std::fclose(f);
  if (!ok) return MPCMD_ERR_CHECKPOINT;
  uint64_t cs = fnv1a(buf.data(), buf.size() * 8, 1469598103934665603ull);
  cs = fnv1a(fl.data(), fl.size() * 4, cs);
  if (h.version >= 2) {
    cs = fnv1a(anc.data(), anc.size() * 8, cs);
    cs = fnv1a(tags.data(), tags.size() * 4, cs);
  }
  if (cs != h.checksum) return MPCMD_ERR_CHECKPOINT;
  int r = upload(buf.data(), buf.data() + n, buf.data() + 2 * n, buf.data() + 3 * n, buf.data() + 4 * n,
                 buf.data() + 5 * n, fl.data(), buf.data() + 6 * n, buf.data() + 6 * n + 3 * ns,
                 buf.data() + 6 * n + 6 * ns);
  if (r) return r;
  if (h.version >= 2 && (r = set_anchors(anc.data()))) return r;
  restart_pending = true;
  if (!tags.empty() && (r = set_owner_tags(tags.data()))) return r;
  cstep = h.cstep;
  time_count = h.time_count;
  last_rebuild = cstep - time_count;
  last_full = last_rebuild;
  return MPCMD_OK;
}

}  // namespace

struct mpcmd_ctx {
  std::unique_ptr<EngineBase> e;
};

extern "C" {

int mpcmd_create(const mpcmd_config* cfg, mpcmd_ctx** out) {
  if (!cfg || !out) return MPCMD_ERR_CONFIG;
  *out = nullptr;
  cudaGetLastError();
  std::unique_ptr<mpcmd_ctx> c(new mpcmd_ctx);
  if (cfg->precision == MPCMD_PREC_FP64) c->e.reset(new Engine<double>());
  else if (cfg->precision == MPCMD_PREC_FP32 || cfg->precision == 0) c->e.reset(new Engine<float>());
  else return MPCMD_ERR_CONFIG;
  int r = c->e->init(*cfg);
  if (r) return r;
  *out = c.release();
  return MPCMD_OK;
}

int mpcmd_destroy(mpcmd_ctx* ctx) {
  delete ctx;
  return MPCMD_OK;
}

const char* mpcmd_error_string(int s) {
  switch (s) {
    case MPCMD_OK: return "ok";
    case MPCMD_ERR_CONFIG: return "invalid configuration";
    case MPCMD_ERR_ALLOC: return "allocation failed";
    case MPCMD_ERR_CELL_OVERFLOW: return "cell capacity exceeded";
    case MPCMD_ERR_NEIGHBOUR_OVERFLOW: return "shell or neighbour capacity exceeded";
    case MPCMD_ERR_RATTLE: return "RATTLE did not converge";
    case MPCMD_ERR_INIT: return "initial placement failed";
    case MPCMD_ERR_STATE: return "call out of order";
    case MPCMD_ERR_CUDA: return cudaGetErrorString(last_cuda);
    case MPCMD_ERR_IO: return "checkpoint i/o failed";
    case MPCMD_ERR_CHECKPOINT: return "checkpoint corrupt or mismatched";
    default: return "unknown status";
  }
}

// Every entry point first clears a stale CUDA error of this thread (left by
// another context or library) so launch errors are attributed to this call.
#define CTX_OK(ctx)                               \
  do {                                            \
    if (!(ctx) || !(ctx)->e) return MPCMD_ERR_STATE; \
    cudaGetLastError();                           \
  } while (0)

int mpcmd_device_bytes(const mpcmd_ctx* ctx, int64_t* bytes) {
  CTX_OK(ctx);
  *bytes = ctx->e->bytes;
  return MPCMD_OK;
}

int mpcmd_upload_state(mpcmd_ctx* ctx, const double* x, const double* y, const double* z, const double* vx,
                       const double* vy, const double* vz, const int32_t* flag, const double* dpos,
                       const double* dvel, const double* dforce) {
  CTX_OK(ctx);
  if (!x || !y || !z || !vx || !vy || !vz || !flag) return MPCMD_ERR_CONFIG;
  if (ctx->e->cfg.n_dimers > 0 && (!dpos || !dvel)) return MPCMD_ERR_CONFIG;
  return ctx->e->upload(x, y, z, vx, vy, vz, flag, dpos, dvel, dforce);
}

int mpcmd_download_state(mpcmd_ctx* ctx, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                         int32_t* flag, double* dpos, double* dvel, double* dforce) {
  CTX_OK(ctx);
  return ctx->e->download(x, y, z, vx, vy, vz, flag, dpos, dvel, dforce);
}

int mpcmd_set_cell_order(mpcmd_ctx* ctx, const int32_t* order, int64_t n) {
  CTX_OK(ctx);
  if (!order) return MPCMD_ERR_CONFIG;
  return ctx->e->set_order(order, n);
}

int mpcmd_set_anchors(mpcmd_ctx* ctx, const double* anchors) {
  CTX_OK(ctx);
  return ctx->e->set_anchors(anchors);
}

int mpcmd_get_anchors(mpcmd_ctx* ctx, double* anchors) {
  CTX_OK(ctx);
  return ctx->e->get_anchors(anchors);
}

int mpcmd_prepare_restart(mpcmd_ctx* ctx) {
  CTX_OK(ctx);
  return ctx->e->prepare_restart();
}

int mpcmd_set_owner_tags(mpcmd_ctx* ctx, const int32_t* type_b) {
  CTX_OK(ctx);
  return ctx->e->set_owner_tags(type_b);
}

int mpcmd_get_owner_tags(mpcmd_ctx* ctx, int32_t* type_b) {
  CTX_OK(ctx);
  return ctx->e->get_owner_tags(type_b);
}

int mpcmd_set_step(mpcmd_ctx* ctx, int64_t cstep, int32_t time_count) {
  CTX_OK(ctx);
  return ctx->e->set_step(cstep, time_count);
}

int mpcmd_set_collision(mpcmd_ctx* ctx, double rot_angle, double mpc_dt, const double* k) {
  CTX_OK(ctx);
  return ctx->e->set_collision(rot_angle, mpc_dt, k);
}

int mpcmd_set_resort(mpcmd_ctx* ctx, int64_t every) {
  CTX_OK(ctx);
  return ctx->e->set_resort(every);
}

int mpcmd_set_reactive_grid(mpcmd_ctx* ctx, const int32_t* table) {
  CTX_OK(ctx);
  return ctx->e->set_reactive_grid(table);
}

int mpcmd_initial(mpcmd_ctx* ctx) { CTX_OK(ctx); return ctx->e->initial(); }
int mpcmd_prepare(mpcmd_ctx* ctx) { CTX_OK(ctx); return ctx->e->prepare(); }
int mpcmd_step(mpcmd_ctx* ctx) { CTX_OK(ctx); return ctx->e->run(1, true); }
int mpcmd_evolve(mpcmd_ctx* ctx) { CTX_OK(ctx); return ctx->e->run(1, false); }
int mpcmd_run(mpcmd_ctx* ctx, int64_t nsteps) { CTX_OK(ctx); return ctx->e->run(nsteps, true); }
int mpcmd_sort(mpcmd_ctx* ctx) { CTX_OK(ctx); return ctx->e->sort_stage(); }
int mpcmd_rebuild_lists(mpcmd_ctx* ctx) { CTX_OK(ctx); return ctx->e->rebuild_stage(); }
int mpcmd_distribute(mpcmd_ctx* ctx) { CTX_OK(ctx); return ctx->e->distribute_stage(); }
int mpcmd_mpc_rotation(mpcmd_ctx* ctx) { CTX_OK(ctx); return ctx->e->rotation_stage(); }
int mpcmd_reaction(mpcmd_ctx* ctx) { CTX_OK(ctx); return ctx->e->reaction_stage(); }
int mpcmd_observables(mpcmd_ctx* ctx, mpcmd_obs* out) {
  CTX_OK(ctx);
  if (!out) return MPCMD_ERR_CONFIG;
  return ctx->e->observables(out);
}
int mpcmd_concentration(mpcmd_ctx* ctx, const mpcmd_conc_params* p, double* totals, double* c1d_a,
                        double* c1d_b, double* xy_a, double* xy_b, double* xz_a, double* xz_b, double* yz_a,
                        double* yz_b) {
  CTX_OK(ctx);
  if (!p) return MPCMD_ERR_CONFIG;
  double* const fields[8] = {c1d_a, c1d_b, xy_a, xy_b, xz_a, xz_b, yz_a, yz_b};
  return ctx->e->concentration(p, totals, fields);
}
int mpcmd_dimer_axes(mpcmd_ctx* ctx, int normalize, double* nucvec, double* vdot) {
  CTX_OK(ctx);
  return ctx->e->dimer_axes(normalize, nucvec, vdot);
}
int mpcmd_checkpoint(mpcmd_ctx* ctx, const char* path) {
  CTX_OK(ctx);
  if (!path) return MPCMD_ERR_CONFIG;
  return ctx->e->checkpoint(path);
}
int mpcmd_restore(mpcmd_ctx* ctx, const char* path) {
  CTX_OK(ctx);
  if (!path) return MPCMD_ERR_CONFIG;
  return ctx->e->restore(path);
}
int mpcmd_get_new_cell(mpcmd_ctx* ctx, int64_t* newcell) { CTX_OK(ctx); return ctx->e->get_new_cell(newcell); }
int mpcmd_get_cell_rotation(mpcmd_ctx* ctx, double* cm, double* axis, int32_t* count) {
  CTX_OK(ctx);
  return ctx->e->get_cell_rotation(cm, axis, count);
}
int mpcmd_get_distribute(mpcmd_ctx* ctx, int32_t* counts, int64_t* first) {
  CTX_OK(ctx);
  return ctx->e->get_distribute(counts, first);
}
int mpcmd_get_affected(mpcmd_ctx* ctx, int32_t* affected) { CTX_OK(ctx); return ctx->e->get_affected(affected); }
int mpcmd_get_shift(mpcmd_ctx* ctx, double* shift) {
  CTX_OK(ctx);
  for (int c = 0; c < 3; ++c) shift[c] = ctx->e->shift[c];
  return MPCMD_OK;
}
int mpcmd_get_pairs(mpcmd_ctx* ctx, int64_t* n_pairs, int64_t* particle, int32_t* sphere) {
  CTX_OK(ctx);
  return ctx->e->get_pairs(n_pairs, particle, sphere);
}
int mpcmd_get_inside(mpcmd_ctx* ctx, int64_t* n_inside, int64_t* idx) {
  CTX_OK(ctx);
  return ctx->e->get_inside(n_inside, idx);
}
int mpcmd_get_counters(mpcmd_ctx* ctx, int64_t* counters, int32_t n) {
  CTX_OK(ctx);
  return ctx->e->get_counters(counters, n);
}
int mpcmd_reactive_grid_table(mpcmd_ctx* ctx, int32_t* table) {
  CTX_OK(ctx);
  for (size_t i = 0; i < ctx->e->react.size(); ++i) table[i] = ctx->e->react[i];
  return MPCMD_OK;
}
int mpcmd_cell_order(mpcmd_ctx* ctx, int32_t* order) {
  CTX_OK(ctx);
  std::memcpy(order, ctx->e->order.data(), ctx->e->order.size() * 4);
  return MPCMD_OK;
}
int64_t mpcmd_kernel_launches(mpcmd_ctx* ctx) {
  (void)ctx;
  return mpcmd::g_kernel_launches;
}
int mpcmd_set_device(int device) {
  if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return MPCMD_ERR_CUDA; }
  return MPCMD_OK;
}
int mpcmd_event_record(mpcmd_ctx* ctx, int slot) { CTX_OK(ctx); return ctx->e->event_record(slot); }
int mpcmd_event_elapsed(mpcmd_ctx* ctx, int a, int b, double* ms) {
  CTX_OK(ctx);
  if (!ms) return MPCMD_ERR_CONFIG;
  return ctx->e->event_elapsed(a, b, ms);
}
int mpcmd_synchronize(mpcmd_ctx* ctx) { CTX_OK(ctx); return ctx->e->synchronize(); }
int mpcmd_profile(mpcmd_ctx* ctx, int enable) { CTX_OK(ctx); return ctx->e->profile(enable); }
int mpcmd_profile_read(mpcmd_ctx* ctx, double* ms, int64_t* count, int n) {
  CTX_OK(ctx);
  if (!ms || !count) return MPCMD_ERR_CONFIG;
  return ctx->e->profile_read(ms, count, n);
}
double mpcmd_contract_u01(uint64_t seed, uint32_t tag, uint32_t index, uint32_t extra, uint32_t step, int which) {
  double u0, u1;
  contract_pair(seed, tag, index, extra, step, u0, u1);
  return which ? u1 : u0;
}

}  // extern "C"
