// Host orchestration of the batched ensemble for one working precision.
// Included once per precision by mpcmd_ensemble_f32.cu / mpcmd_ensemble_f64.cu.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mpcmd_engine.cuh"
#include "mpcmd_ensemble.cuh"
#include "mpcmd_ensemble_base.h"

namespace mpcmd {
namespace ens {

#define ECK(call)                          \
  do {                                     \
    cudaError_t e_ = (call);               \
    if (e_ != cudaSuccess) return MPCMD_ERR_CUDA; \
  } while (0)

constexpr double kPiE = 3.141592653589793;

template <typename T>
struct Ensemble : EnsembleBase {
  mpcmd_ensemble_config cfg{};
  std::vector<mpcmd_replica> reps;
  std::vector<Rep<T>> hrep;
  int R = 0, P = 0, rattle_max = 100000;
  int64_t ntot = 0, ctot = 0, stot = 0, max_n = 0;
  EDev<T> d{};
  std::vector<void*> allocs;
  uint32_t* scan_tmp = nullptr;
  double* d_mass = nullptr;
  double* d_obs = nullptr;
  double* staging = nullptr;
  int32_t* staging_i = nullptr;
  void* tile_mem[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  cudaStream_t st = nullptr;
  cudaEvent_t ev[8] = {};
  cudaGraphExec_t gexec = nullptr;
  int64_t graph_launches = 0;
  int tile = 2048, block = 256, sblock = 256;
  int g_part = 0, g_shell = 0, nsm = 0;
  int64_t cstep = 0;
  bool prepared = false, need_advance = true, vel_pending = false;
  int64_t launches = 0, replays = 0, field_samples = 0;
  // tuner snapshot
  std::vector<std::pair<void*, size_t>> snap_regions;   // (device source, bytes)
  std::vector<void*> snap_copies;
  int64_t snap_cstep = 0;
  bool snap_prepared = false, snap_need_advance = true, snap_vel_pending = false;

  ~Ensemble() override {
    if (gexec) cudaGraphExecDestroy(gexec);
    release_snapshot();
    if (d.axes) cudaFree(d.axes);
    if (d.field) cudaFree(d.field);
    for (void* p : tile_mem) if (p) cudaFree(p);
    for (void* p : allocs) cudaFree(p);
    for (cudaEvent_t e : ev) if (e) cudaEventDestroy(e);
    if (st) cudaStreamDestroy(st);
  }

  template <class U>
  int alloc(U*& p, int64_t n) {
    void* q = nullptr;
    const size_t b = sizeof(U) * (size_t)std::max<int64_t>(n, 1);
    if (cudaMalloc(&q, b) != cudaSuccess) return MPCMD_ERR_ALLOC;
    allocs.push_back(q);
    bytes += (int64_t)b;
    p = static_cast<U*>(q);
    return MPCMD_OK;
  }

  static void fill_params(const mpcmd_replica& rp, const mpcmd_ensemble_config& c, KParams<T>& kp) {
    std::memset(&kp, 0, sizeof(kp));
    kp.lx = rp.lx; kp.ly = rp.ly; kp.lz = rp.lz;
    kp.geometry = MPCMD_GEOM_PERIODIC; kp.ns = 2; kp.nd = 1;
    kp.catalysis = MPCMD_CAT_DETERMINISTIC; kp.exclusion = MPCMD_EXCL_PARTICLE;
    kp.kinetics = MPCMD_KIN_SIMPLE; kp.rotation_sense = 1;
    kp.react_dir = 0; kp.cell_capacity = c.cell_capacity;
    kp.n = rp.n_solvent;
    kp.ncell = (int64_t)rp.lx * rp.ly * rp.lz;
    kp.ncell_shift = kp.ncell;
    kp.seed = rp.seed;
    kp.Lx = (T)rp.lx; kp.Ly = (T)rp.ly; kp.Lz = (T)rp.lz;
    kp.Ld[0] = rp.lx; kp.Ld[1] = rp.ly; kp.Ld[2] = rp.lz;
    kp.dt = (T)c.md_dt; kp.dtd = c.md_dt;
    for (int s = 0; s < 4; ++s) {
      kp.hIM[s] = (T)((0.5 * c.md_dt) / rp.mass[s]);
      kp.eps_c[s] = (T)rp.eps_c[s];
      kp.eps_n[s] = (T)rp.eps_n[s];
    }
    const double cut = std::pow(2.0, 1.0 / 6.0);
    const double Rr[2] = {rp.rc, rp.rn};
    for (int t = 0; t < 2; ++t) {
      const double co = Rr[t] * cut;
      kp.cut2[t] = (T)(co * co);
      kp.cut2_strict[t] = (T)(co * co);
      kp.full2[t] = (T)((co + c.skin) * (co + c.skin));
      const double r2 = Rr[t] * Rr[t], R6 = r2 * r2 * r2, R12 = R6 * R6;
      kp.R6[t] = (T)R6; kp.R12[t] = (T)R12; kp.r6R6[t] = (T)(6.0 * R6); kp.r12R12[t] = (T)(12.0 * R12);
    }
    kp.msd_thr = (T)((0.5 * c.skin) * (0.5 * c.skin));
    kp.cosrot = (T)std::cos(c.rot_angle);
    kp.sinrot = (T)std::sin(c.rot_angle);
    kp.tau = c.mpc_dt;
    kp.k[0] = rp.k1; kp.kf[0] = (float)rp.k1;
    kp.tauf = (float)c.mpc_dt;
    kp.mc = rp.mc; kp.mn = rp.mn; kp.dcn = rp.dcn;
    kp.hIMc = (0.5 * c.md_dt) / rp.mc; kp.hIMn = (0.5 * c.md_dt) / rp.mn;
    kp.IIM = 1.0 / ((1.0 / rp.mc) + (1.0 / rp.mn));
    kp.iMc = 1.0 / rp.mc; kp.iMn = 1.0 / rp.mn; kp.iD2 = 1.0 / (rp.dcn * rp.dcn);
    kp.iMcdt = 1.0 / (rp.mc * c.md_dt); kp.iMndt = 1.0 / (rp.mn * c.md_dt);
  }

  int create(const mpcmd_ensemble_config& c, const mpcmd_replica* rp) {
    cfg = c;
    R = c.n_replicas;
    if (R <= 0 || R > (1 << 20) || !rp) return MPCMD_ERR_CONFIG;
    if (!(c.md_dt > 0) || !(c.mpc_dt > 0) || !(c.skin > 0)) return MPCMD_ERR_CONFIG;
    P = (int)std::lround(c.mpc_dt / c.md_dt);
    if (P < 1 || std::fabs(P * c.md_dt - c.mpc_dt) > 1e-9 * c.mpc_dt) return MPCMD_ERR_CONFIG;
    if (c.sort_every < 0 || (c.sort_every > 0 && c.sort_every % P != 0)) return MPCMD_ERR_CONFIG;
    if (c.cell_capacity < 1 || c.cell_capacity > 255) return MPCMD_ERR_CONFIG;
    rattle_max = c.rattle_max_iter > 0 ? c.rattle_max_iter : 100000;
    reps.assign(rp, rp + R);
    const double cut = std::pow(2.0, 1.0 / 6.0);
    hrep.resize(R);
    for (int r = 0; r < R; ++r) {
      mpcmd_replica& q = reps[r];
      if (q.lx < 4 || q.ly < 4 || q.lz < 4 || q.lx > 1024 || q.ly > 1024 || q.lz > 1024) return MPCMD_ERR_CONFIG;
      if (q.n_solvent <= 0) return MPCMD_ERR_CONFIG;
      if (!(q.rc > 0) || !(q.rn > 0) || !(q.dcn > 0) || !(q.kT > 0) || !(q.k1 >= 0)) return MPCMD_ERR_CONFIG;
      for (int s = 0; s < 4; ++s)
        if (!(q.mass[s] > 0)) return MPCMD_ERR_CONFIG;
      const double half = 0.5 * std::min(q.lx, std::min(q.ly, q.lz));
      // minimum images of the bond and of the list radii must be unique
      if (q.dcn >= half || q.rc * cut + c.skin >= half || q.rn * cut + c.skin >= half) return MPCMD_ERR_CONFIG;
      const int64_t ncell = (int64_t)q.lx * q.ly * q.lz;
      if (q.mc <= 0 || q.mn <= 0) {   // main_pattern.f95:118-119
        const double rho = (double)q.n_solvent / (double)ncell;
        q.mc = rho * ((4.0 * kPiE) / 3) * q.rc * q.rc * q.rc;
        q.mn = rho * ((4.0 * kPiE) / 3) * q.rn * q.rn * q.rn;
      }
      Rep<T>& h = hrep[r];
      std::memset(&h, 0, sizeof(h));
      fill_params(q, c, h.kp);
      h.poff = ntot; h.n = q.n_solvent;
      h.coff = ctot;
      const double rho = (double)q.n_solvent / (double)ncell;
      const double vc = 4.0 / 3.0 * kPiE * std::pow(q.rc * cut + c.skin + 1.0, 3);
      const double vn = 4.0 / 3.0 * kPiE * std::pow(q.rn * cut + c.skin + 1.0, 3);
      h.scap = (int64_t)std::min<double>((double)q.n_solvent, (vc + vn) * rho * 1.5 + 1024.0);
      h.soff = stot;
      h.skin = c.skin;
      h.mcn = q.mc + q.mn;
      for (int s = 0; s < 4; ++s) h.sd[s] = std::sqrt(q.kT / q.mass[s]);
      ntot += q.n_solvent; ctot += ncell; stot += h.scap;
      max_n = std::max<int64_t>(max_n, q.n_solvent);
    }
    if (ntot >= (int64_t)1 << 31 || ctot >= (int64_t)1 << 32) return MPCMD_ERR_CONFIG;

    int dev = 0;
    ECK(cudaGetDevice(&dev));
    ECK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    ECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    for (cudaEvent_t& e : ev) ECK(cudaEventCreate(&e));

    int s = 0;
    s |= alloc(d.cell, ntot); s |= alloc(d.ox, ntot); s |= alloc(d.oy, ntot); s |= alloc(d.oz, ntot);
    s |= alloc(d.vx, ntot); s |= alloc(d.vy, ntot); s |= alloc(d.vz, ntot); s |= alloc(d.flag, ntot);
    s |= alloc(d.pkey, ntot);
    s |= alloc(d.cell2, ntot); s |= alloc(d.ox2, ntot); s |= alloc(d.oy2, ntot); s |= alloc(d.oz2, ntot);
    s |= alloc(d.vx2, ntot); s |= alloc(d.vy2, ntot); s |= alloc(d.vz2, ntot); s |= alloc(d.flag2, ntot);
    s |= alloc(d.sidx, ntot);
    s |= alloc(d.sh_idx, stot); s |= alloc(d.sh_mask, stot); s |= alloc(d.sh_fp, 6 * stot); s |= alloc(d.sh_msd, stot);
    T* rot = nullptr;
    s |= alloc(rot, 6 * ctot);
    d.rot = rot;
    if (sizeof(T) == 4) { float4* a = nullptr; s |= alloc(a, ctot); d.acc = a; }
    else { double* a = nullptr; s |= alloc(a, 4 * ctot); d.acc = a; }
    s |= alloc(d.dcnt, ctot); s |= alloc(d.dfirst, 4 * ctot); s |= alloc(d.order_rank, ctot);
    s |= alloc(d.scnt, ctot); s |= alloc(d.sstart, ctot); s |= alloc(d.sfill, ctot);
    s |= alloc(scan_tmp, scan_tmp_words(ctot));
    Rep<T>* drep = nullptr; Dyn<T>* ddyn = nullptr; Glob* dg = nullptr;
    s |= alloc(drep, R); s |= alloc(ddyn, R); s |= alloc(dg, 1);
    s |= alloc(d.st_prefix, R + 1);
    s |= alloc(d.rt_prefix, R + 1);
    s |= alloc(d_mass, 4 * (int64_t)R); s |= alloc(d_obs, 8 * (int64_t)R);
    if (s) return MPCMD_ERR_ALLOC;
    d.rep = drep; d.dyn = ddyn; d.g = dg; d.R = R; d.mpc_every = P;
    ECK(cudaMemcpyAsync(drep, hrep.data(), sizeof(Rep<T>) * R, cudaMemcpyHostToDevice, st));
    ECK(cudaMemsetAsync(ddyn, 0, sizeof(Dyn<T>) * R, st));
    ECK(cudaMemsetAsync(dg, 0, sizeof(Glob), st));
    ECK(cudaMemsetAsync(d.st_prefix, 0, sizeof(uint32_t) * (R + 1), st));
    ECK(cudaMemsetAsync(d.rt_prefix, 0, sizeof(uint32_t) * (R + 1), st));
    ECK(cudaMemsetAsync(d.acc, 0, (sizeof(T) == 4 ? 16 : 32) * (size_t)ctot, st));
    ECK(cudaMemsetAsync(d.dcnt, 0, 4 * (size_t)ctot, st));
    ECK(cudaMemsetAsync(d.dfirst, 0xFF, 16 * (size_t)ctot, st));
    ECK(cudaMemsetAsync(d.flag, 0, (size_t)ntot, st));
    std::vector<uint32_t> rank((size_t)ctot);
    std::vector<double> mass(4 * (size_t)R);
    for (int r = 0; r < R; ++r) {
      const std::vector<int32_t> ord = default_cell_order(reps[r].lx, reps[r].ly, reps[r].lz);
      for (size_t k = 0; k < ord.size(); ++k) rank[(size_t)hrep[r].coff + (size_t)ord[k]] = (uint32_t)k;
      for (int q = 0; q < 4; ++q) mass[4 * (size_t)r + q] = reps[r].mass[q];
    }
    ECK(cudaMemcpyAsync(d.order_rank, rank.data(), 4 * (size_t)ctot, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(d_mass, mass.data(), 8 * mass.size(), cudaMemcpyHostToDevice, st));
    ECK(cudaStreamSynchronize(st));
    int r = set_schedule(c.particle_tile > 0 ? c.particle_tile : 2048, c.block > 0 ? c.block : 256,
                         c.shell_block > 0 ? c.shell_block : 256);
    return r;
  }

  // ---------------------------------------------------------- schedule --
  int set_schedule(int pt, int b, int sb) override {
    if (pt < 64 || pt > (1 << 20) || b < 32 || b > MAX_BLOCK || b % 32 || sb < 32 || sb > MAX_BLOCK || sb % 32)
      return MPCMD_ERR_CONFIG;
    tile = pt; block = b; sblock = sb;
    d.tile = pt;
    std::vector<uint32_t> prep, crep;
    std::vector<int64_t> plo, phi, clo, chi;
    for (int r = 0; r < R; ++r) {
      for (int64_t lo = 0; lo < hrep[r].n; lo += pt) {
        prep.push_back((uint32_t)r);
        plo.push_back(hrep[r].poff + lo);
        phi.push_back(hrep[r].poff + std::min<int64_t>(lo + pt, hrep[r].n));
      }
      for (int64_t lo = 0; lo < hrep[r].kp.ncell; lo += pt) {
        crep.push_back((uint32_t)r);
        clo.push_back(lo);
        chi.push_back(std::min<int64_t>(lo + pt, hrep[r].kp.ncell));
      }
    }
    ECK(cudaStreamSynchronize(st));
    for (void*& p : tile_mem) { if (p) cudaFree(p); p = nullptr; }
    const size_t np = prep.size(), nc = crep.size();
    ECK(cudaMalloc(&tile_mem[0], 4 * np)); ECK(cudaMalloc(&tile_mem[1], 8 * np)); ECK(cudaMalloc(&tile_mem[2], 8 * np));
    ECK(cudaMalloc(&tile_mem[3], 4 * nc)); ECK(cudaMalloc(&tile_mem[4], 8 * nc)); ECK(cudaMalloc(&tile_mem[5], 8 * nc));
    ECK(cudaMemcpyAsync(tile_mem[0], prep.data(), 4 * np, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(tile_mem[1], plo.data(), 8 * np, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(tile_mem[2], phi.data(), 8 * np, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(tile_mem[3], crep.data(), 4 * nc, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(tile_mem[4], clo.data(), 8 * nc, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(tile_mem[5], chi.data(), 8 * nc, cudaMemcpyHostToDevice, st));
    ECK(cudaStreamSynchronize(st));
    d.pt_rep = (const uint32_t*)tile_mem[0]; d.pt_lo = (const int64_t*)tile_mem[1]; d.pt_hi = (const int64_t*)tile_mem[2];
    d.ct_rep = (const uint32_t*)tile_mem[3]; d.ct_lo = (const int64_t*)tile_mem[4]; d.ct_hi = (const int64_t*)tile_mem[5];
    d.n_ptiles = (int)np; d.n_ctiles = (int)nc;
    int occ_p = 0, occ_s = 0;
    ECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_p, k_ens_rebuild<T>, b, 0));
    ECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, k_ens_force<T>, sb, 0));
    g_part = nsm * std::max(occ_p, 1);
    g_shell = nsm * std::max(occ_s, 1);
    invalidate_graph();
    return MPCMD_OK;
  }

  void get_schedule(int* s) const override { s[0] = tile; s[1] = block; s[2] = sblock; }

  void invalidate_graph() {
    if (gexec) { cudaGraphExecDestroy(gexec); gexec = nullptr; }
  }

  // ---------------------------------------------------------- launches --
  void L_force(int mode) { k_ens_force<T><<<g_shell, sblock, 0, st>>>(d, mode); ++launches; }
  void L_dimer(int mode) {
    if (sizeof(T) == 4) {
      // four lanes per replica, one 32-lane block per eight replicas (spread over the SMs)
      k_ens_dimer_split<T><<<(4 * R + 31) / 32, 32, 0, st>>>(d, mode, rattle_max);
    } else {
      k_ens_dimer<T><<<(R + 127) / 128, 128, 0, st>>>(d, mode, rattle_max);
    }
    ++launches;
  }
  void L_plan() { k_ens_plan<T><<<1, 1024, 0, st>>>(d); ++launches; }
  void L_rebuild(int mode) { k_ens_rebuild<T><<<g_part, block, 0, st>>>(d, mode); ++launches; }
  void L_finalize(int adv) { k_ens_finalize<T><<<1, 1024, 0, st>>>(d, sblock, adv); ++launches; }
  void L_sort() {
    const int g = nsm * 8;
    cudaMemsetAsync(d.scnt, 0, 4 * (size_t)ctot, st);
    cudaMemsetAsync(d.sfill, 0, 4 * (size_t)ctot, st);
    k_ens_sort_count<T><<<g_part, block, 0, st>>>(d);
    scan_u32(d.scnt, d.sstart, ctot, scan_tmp, st);
    k_ens_sort_fill<T><<<g_part, block, 0, st>>>(d);
    k_ens_sort_segments<T><<<g, 256, 0, st>>>(d, ctot);
    k_ens_sort_gather<T><<<g, 256, 0, st>>>(d, ntot);
    // back into the main arrays, so that every kernel argument stays valid
    cudaMemcpyAsync(d.cell, d.cell2, 4 * (size_t)ntot, cudaMemcpyDeviceToDevice, st);
    T* src[6] = {d.ox2, d.oy2, d.oz2, d.vx2, d.vy2, d.vz2};
    T* dst[6] = {d.ox, d.oy, d.oz, d.vx, d.vy, d.vz};
    for (int q = 0; q < 6; ++q) cudaMemcpyAsync(dst[q], src[q], sizeof(T) * (size_t)ntot, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(d.flag, d.flag2, (size_t)ntot, cudaMemcpyDeviceToDevice, st);
    launches += 5;
  }

  bool sort_step(int64_t s) const { return cfg.sort_every > 0 && s % cfg.sort_every == 0; }

  // One main-loop iteration of every replica (the step cstep + 1).  `last`:
  // no step follows in this call, so the next step's first kick and free
  // flight are left to the next call.
  void issue_step(bool last) {
    const int64_t s = cstep + 1;
    const bool mpc = s % P == 0;
    if (need_advance) { L_force(M_ADVANCE); need_advance = false; }
    L_dimer((vel_pending ? M_VEL : 0) | M_POS);
    vel_pending = false;
    L_plan();
    if (sort_step(s)) {
      L_rebuild(M_LAZY);
      L_sort();
      L_rebuild(M_LISTS);
    } else {
      L_rebuild(M_LAZY | M_LISTS);
    }
    L_finalize(1);
    if (mpc) {
      L_force(M_FORCE);
      L_dimer(M_VEL);
      k_ens_collide<T><<<g_part, block, 0, st>>>(d);
      k_ens_cells<T><<<g_part, block, 0, st>>>(d);
      k_ens_rotate<T><<<g_part, block, 0, st>>>(d);
      launches += 3;
      need_advance = true;
    } else if (last) {
      L_force(M_FORCE);
      vel_pending = true;
      need_advance = true;
    } else {
      L_force(M_FORCE | M_ADVANCE);
      vel_pending = true;
    }
    cstep = s;
  }

  int capture_period() {
    invalidate_graph();
    const int64_t c0 = cstep, l0 = launches;
    cudaGraph_t g = nullptr;
    ECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < P; ++k) issue_step(k == P - 1);
    cudaError_t e = cudaStreamEndCapture(st, &g);
    cstep = c0;
    graph_launches = launches - l0;
    launches = l0;
    if (e != cudaSuccess) return MPCMD_ERR_CUDA;
    e = cudaGraphInstantiate(&gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { gexec = nullptr; return MPCMD_ERR_CUDA; }
    return MPCMD_OK;
  }

  int check_status() {
    ECK(cudaStreamSynchronize(st));
    ECK(cudaGetLastError());
    std::vector<Dyn<T>> h(R);
    ECK(cudaMemcpy(h.data(), d.dyn, sizeof(Dyn<T>) * R, cudaMemcpyDeviceToHost));
    int any = 0;
    for (int r = 0; r < R; ++r) any |= h[r].status;
    if (any & E_ERR_INIT) return MPCMD_ERR_INIT;
    if (any & E_ERR_RATTLE) return MPCMD_ERR_RATTLE;
    if (any & E_ERR_SHELL) return MPCMD_ERR_NEIGHBOUR_OVERFLOW;
    if (any & E_ERR_CELL) return MPCMD_ERR_CELL_OVERFLOW;
    return MPCMD_OK;
  }

  int run(int64_t n) override {
    if (!prepared) return MPCMD_ERR_STATE;
    if (n < 0) return MPCMD_ERR_CONFIG;
    int64_t done = 0;
    while (done < n) {
      const bool graphable = cstep % P == 0 && need_advance && !vel_pending && n - done >= P;
      bool sort_inside = false;
      for (int64_t s = cstep + 1; s <= cstep + P && graphable; ++s) sort_inside |= sort_step(s);
      if (graphable && !sort_inside) {
        if (!gexec) {
          int r = capture_period();
          if (r) return r;
        }
        ECK(cudaGraphLaunch(gexec, st));
        cstep += P;
        done += P;
        replays++;
        launches += graph_launches;
      } else {
        issue_step(done + 1 == n);
        done++;
      }
    }
    if (vel_pending) { L_dimer(M_VEL); vel_pending = false; }
    return check_status();
  }

  // ----------------------------------------------------------- state ----
  int read_dyn(std::vector<Dyn<T>>& h) {
    h.resize(R);
    ECK(cudaStreamSynchronize(st));
    ECK(cudaMemcpy(h.data(), d.dyn, sizeof(Dyn<T>) * R, cudaMemcpyDeviceToHost));
    return MPCMD_OK;
  }
  int write_dyn(const std::vector<Dyn<T>>& h) {
    ECK(cudaMemcpyAsync(d.dyn, h.data(), sizeof(Dyn<T>) * R, cudaMemcpyHostToDevice, st));
    ECK(cudaStreamSynchronize(st));
    return MPCMD_OK;
  }

  static void set_rel(Dyn<T>& y) {
    for (int i = 0; i < 2; ++i) {
      const double* X = y.dpos + 3 * i;
      const double fx = std::floor(X[0]), fy = std::floor(X[1]), fz = std::floor(X[2]);
      y.srel[i].cx = (int)fx; y.srel[i].cy = (int)fy; y.srel[i].cz = (int)fz;
      y.srel[i].ox = (T)(X[0] - fx); y.srel[i].oy = (T)(X[1] - fy); y.srel[i].oz = (T)(X[2] - fz);
    }
  }

  int initial() override {
    // initial_mod.f95:78-119 for one dimer in a periodic box: the first draw
    // of the contract stream places it (no wall and no other dimer rejects it)
    std::vector<Dyn<T>> h;
    int r = read_dyn(h);
    if (r) return r;
    for (int q = 0; q < R; ++q) {
      const mpcmd_replica& rp = reps[q];
      const double L[3] = {(double)rp.lx, (double)rp.ly, (double)rp.lz};
      double ux, uy, uz, uphi, uth, unused;
      contract_pair(rp.seed, TAG_INIT_DIMER, 0, 0, 0, ux, uy);
      contract_pair(rp.seed, TAG_INIT_DIMER, 0, 0, 1, uz, uphi);
      contract_pair(rp.seed, TAG_INIT_DIMER, 0, 0, 2, uth, unused);
      const double phi = 2.0 * kPiE * uphi, theta = 2.0 * uth - 1.0;
      const double sn = std::sqrt(1.0 - theta * theta);
      double Pp[2][3] = {{L[0] * ux + 0.5 * rp.dcn * (sn * std::cos(phi)), L[1] * uy + 0.5 * rp.dcn * (sn * std::sin(phi)),
                          L[2] * uz + 0.5 * rp.dcn * theta},
                         {L[0] * ux - 0.5 * rp.dcn * (sn * std::cos(phi)), L[1] * uy - 0.5 * rp.dcn * (sn * std::sin(phi)),
                          L[2] * uz - 0.5 * rp.dcn * theta}};
      Dyn<T>& y = h[q];
      std::memset(&y, 0, sizeof(y));
      for (int u = 0; u < 2; ++u)
        for (int c = 0; c < 3; ++c) y.dpos[3 * u + c] = Pp[u][c] - L[c] * std::floor(Pp[u][c] / L[c]);
      set_rel(y);
    }
    r = write_dyn(h);
    if (r) return r;
    k_ens_init<T><<<g_part, block, 0, st>>>(d);
    k_ens_sub_mean<T><<<g_part, block, 0, st>>>(d);
    launches += 2;
    cstep = 0;
    prepared = false;
    ECK(cudaMemsetAsync(d.g, 0, sizeof(Glob), st));
    return check_status();
  }

  int ensure_staging() {
    if (staging) return MPCMD_OK;
    int s = alloc(staging, 6 * max_n);
    s |= alloc(staging_i, max_n);
    return s ? MPCMD_ERR_ALLOC : MPCMD_OK;
  }

  int upload(int r, const double* x, const double* y, const double* z, const double* vx, const double* vy,
             const double* vz, const int32_t* flag, const double* dpos, const double* dvel,
             const double* dforce) override {
    if (r < 0 || r >= R || !x || !y || !z || !vx || !vy || !vz || !flag || !dpos) return MPCMD_ERR_CONFIG;
    int s = ensure_staging();
    if (s) return s;
    const int64_t n = hrep[r].n;
    const double* src[6] = {x, y, z, vx, vy, vz};
    for (int q = 0; q < 6; ++q) ECK(cudaMemcpyAsync(staging + q * n, src[q], 8 * (size_t)n, cudaMemcpyHostToDevice, st));
    ECK(cudaMemcpyAsync(staging_i, flag, 4 * (size_t)n, cudaMemcpyHostToDevice, st));
    k_ens_upload<T><<<nsm * 4, 256, 0, st>>>(d, hrep[r].poff, n, reps[r].lx, reps[r].ly, reps[r].lz, staging,
                                             staging + n, staging + 2 * n, staging + 3 * n, staging + 4 * n,
                                             staging + 5 * n, staging_i);
    ++launches;
    std::vector<Dyn<T>> h;
    s = read_dyn(h);
    if (s) return s;
    Dyn<T>& q = h[r];
    for (int c = 0; c < 6; ++c) {
      q.dpos[c] = dpos[c];
      q.dvel[c] = dvel ? dvel[c] : 0.0;
      q.dfrc[c] = dforce ? dforce[c] : 0.0;
    }
    set_rel(q);
    s = write_dyn(h);
    if (s) return s;
    prepared = false;
    return MPCMD_OK;
  }

  int download(int r, double* x, double* y, double* z, double* vx, double* vy, double* vz, int32_t* flag,
               double* dpos, double* dvel, double* dforce) override {
    if (r < 0 || r >= R) return MPCMD_ERR_CONFIG;
    int s = ensure_staging();
    if (s) return s;
    const int64_t n = hrep[r].n;
    k_ens_download<T><<<nsm * 4, 256, 0, st>>>(d, hrep[r].poff, n, staging, staging + n, staging + 2 * n,
                                               staging + 3 * n, staging + 4 * n, staging + 5 * n, staging_i);
    ++launches;
    double* dst[6] = {x, y, z, vx, vy, vz};
    for (int q = 0; q < 6; ++q)
      if (dst[q]) ECK(cudaMemcpyAsync(dst[q], staging + q * n, 8 * (size_t)n, cudaMemcpyDeviceToHost, st));
    if (flag) ECK(cudaMemcpyAsync(flag, staging_i, 4 * (size_t)n, cudaMemcpyDeviceToHost, st));
    std::vector<Dyn<T>> h;
    s = read_dyn(h);
    if (s) return s;
    for (int c = 0; c < 6; ++c) {
      if (dpos) dpos[c] = h[r].dpos[c];
      if (dvel) dvel[c] = h[r].dvel[c];
      if (dforce) dforce[c] = h[r].dfrc[c];
    }
    return MPCMD_OK;
  }

  int prepare() override {
    // main_pattern.f95:168-187 for every replica
    std::vector<Dyn<T>> h;
    int r = read_dyn(h);
    if (r) return r;
    for (Dyn<T>& y : h) {
      y.rebuild = 1; y.n_shell = 0; y.maxv2 = 0ull; y.maxmsd = 0ull; y.time_count = 0;
      for (double& f : y.facc) f = 0.;
    }
    r = write_dyn(h);
    if (r) return r;
    Glob g{};
    g.cstep = (unsigned)cstep;
    ECK(cudaMemcpyAsync(d.g, &g, sizeof(g), cudaMemcpyHostToDevice, st));
    if (sort_step(cstep)) L_sort();
    L_plan();
    L_rebuild(M_LISTS);
    L_finalize(0);
    need_advance = true;
    vel_pending = false;
    prepared = true;
    return check_status();
  }

  int observables(mpcmd_obs* out) override {
    if (!out) return MPCMD_ERR_CONFIG;
    ECK(cudaMemsetAsync(d_obs, 0, 8 * 8 * (size_t)R, st));
    k_ens_observables<T><<<g_part, block, 0, st>>>(d, d_mass, d_obs);
    ++launches;
    std::vector<double> o(8 * (size_t)R);
    ECK(cudaMemcpyAsync(o.data(), d_obs, 8 * o.size(), cudaMemcpyDeviceToHost, st));
    std::vector<Dyn<T>> h;
    int r = read_dyn(h);
    if (r) return r;
    for (int q = 0; q < R; ++q) {
      mpcmd_obs& b = out[q];
      std::memset(&b, 0, sizeof(b));
      const Dyn<T>& y = h[q];
      const double m[2] = {reps[q].mc, reps[q].mn};
      double pd[3] = {0, 0, 0}, ked = 0;
      for (int s = 0; s < 2; ++s)
        for (int c = 0; c < 3; ++c) {
          pd[c] += m[s] * y.dvel[3 * s + c];
          ked += 0.5 * m[s] * y.dvel[3 * s + c] * y.dvel[3 * s + c];
        }
      for (int c = 0; c < 3; ++c) {
        b.solvent_momentum[c] = o[8 * q + c];
        b.momentum[c] = o[8 * q + c] + pd[c];
      }
      b.kinetic_solvent = o[8 * q + 3];
      b.kinetic_dimer = ked;
      b.potential = y.pot;
      for (int s = 0; s < 4; ++s) b.species_count[s] = (int64_t)std::llround(o[8 * q + 4 + s]);
      b.n_inside = y.n_shell;
      b.n_pairs = y.n_shell;
      b.time_count = y.time_count;
      b.time_penetrate = y.time_penetrate;
      b.cstep = cstep;
    }
    return MPCMD_OK;
  }

  // ---------------------------------------------------------- samples --
  int reset_samples(int history) override {
    if (history < 0) return MPCMD_ERR_CONFIG;
    ECK(cudaStreamSynchronize(st));
    if (d.axes) { cudaFree(d.axes); d.axes = nullptr; }
    d.hist = 0;
    if (history > 0) {
      ECK(cudaMalloc(&d.axes, sizeof(float) * 3 * (size_t)history * R));
      ECK(cudaMemsetAsync(d.axes, 0, sizeof(float) * 3 * (size_t)history * R, st));
      d.hist = history;
    }
    std::vector<Dyn<T>> h;
    int r = read_dyn(h);
    if (r) return r;
    for (Dyn<T>& y : h) { y.vdot_sum = 0.; y.vdot_n = 0; }
    r = write_dyn(h);
    invalidate_graph();
    return r;
  }

  int samples(double* mean, int64_t* count, float* axes) override {
    std::vector<Dyn<T>> h;
    int r = read_dyn(h);
    if (r) return r;
    for (int q = 0; q < R; ++q) {
      if (mean) mean[q] = h[q].vdot_n ? h[q].vdot_sum / (double)h[q].vdot_n : 0.0;
      if (count) count[q] = h[q].vdot_n;
    }
    if (axes && d.axes && d.hist > 0)
      ECK(cudaMemcpy(axes, d.axes, sizeof(float) * 3 * (size_t)d.hist * R, cudaMemcpyDeviceToHost));
    return MPCMD_OK;
  }

  int field_accumulate(int nz, int nr, double zmax, double rmax) override {
    if (nz <= 0 || nr <= 0 || nz * nr > (1 << 20) || !(zmax > 0) || !(rmax > 0)) return MPCMD_ERR_CONFIG;
    if (nz != d.nz || nr != d.nr || (float)zmax != d.zmax || (float)rmax != d.rmax || !d.field) {
      ECK(cudaStreamSynchronize(st));
      if (d.field) cudaFree(d.field);
      ECK(cudaMalloc(&d.field, sizeof(uint32_t) * (size_t)nz * nr * R));
      ECK(cudaMemsetAsync(d.field, 0, sizeof(uint32_t) * (size_t)nz * nr * R, st));
      d.nz = nz; d.nr = nr; d.zmax = (float)zmax; d.rmax = (float)rmax;
      field_samples = 0;
      invalidate_graph();
    }
    k_ens_field<T><<<g_part, block, 0, st>>>(d);
    ++launches;
    field_samples++;
    return MPCMD_OK;
  }

  int field_read(uint32_t* counts, int64_t* nsamp) override {
    if (!d.field) return MPCMD_ERR_STATE;
    ECK(cudaStreamSynchronize(st));
    if (counts) ECK(cudaMemcpy(counts, d.field, sizeof(uint32_t) * (size_t)d.nz * d.nr * R, cudaMemcpyDeviceToHost));
    if (nsamp) *nsamp = field_samples;
    return MPCMD_OK;
  }

  // ---------------------------------------------------------- snapshot --
  int snapshot(bool save) override {
    ECK(cudaStreamSynchronize(st));
    if (save) {
      release_snapshot();
      snap_regions = {{d.cell, 4 * (size_t)ntot}, {d.ox, sizeof(T) * (size_t)ntot}, {d.oy, sizeof(T) * (size_t)ntot},
                      {d.oz, sizeof(T) * (size_t)ntot}, {d.vx, sizeof(T) * (size_t)ntot},
                      {d.vy, sizeof(T) * (size_t)ntot}, {d.vz, sizeof(T) * (size_t)ntot}, {d.flag, (size_t)ntot},
                      {d.sh_idx, 4 * (size_t)stot}, {d.sh_mask, (size_t)stot}, {d.sh_fp, 6 * sizeof(T) * (size_t)stot},
                      {d.sh_msd, sizeof(T) * (size_t)stot}, {d.dyn, sizeof(Dyn<T>) * (size_t)R},
                      {d.g, sizeof(Glob)}, {d.st_prefix, 4 * (size_t)(R + 1)},
                      {d.rt_prefix, 4 * (size_t)(R + 1)}};
      for (auto& rg : snap_regions) {
        void* p = nullptr;
        if (cudaMalloc(&p, rg.second) != cudaSuccess) { release_snapshot(); return MPCMD_ERR_ALLOC; }
        snap_copies.push_back(p);
        ECK(cudaMemcpyAsync(p, rg.first, rg.second, cudaMemcpyDeviceToDevice, st));
      }
      snap_cstep = cstep; snap_prepared = prepared; snap_need_advance = need_advance; snap_vel_pending = vel_pending;
    } else {
      if (snap_copies.size() != snap_regions.size() || snap_copies.empty()) return MPCMD_ERR_STATE;
      for (size_t k = 0; k < snap_regions.size(); ++k)
        ECK(cudaMemcpyAsync(snap_regions[k].first, snap_copies[k], snap_regions[k].second, cudaMemcpyDeviceToDevice, st));
      cstep = snap_cstep; prepared = snap_prepared; need_advance = snap_need_advance; vel_pending = snap_vel_pending;
    }
    ECK(cudaStreamSynchronize(st));
    return MPCMD_OK;
  }

  void release_snapshot() override {
    for (void* p : snap_copies) cudaFree(p);
    snap_copies.clear();
    snap_regions.clear();
  }

  bool at_period_boundary() const override { return prepared && cstep % P == 0 && need_advance && !vel_pending; }
  int mpc_every() const override { return P; }

  std::string shape_class() const override {
    // precision, replica count and total particle count, each rounded to a
    // power of two: ensembles in one class share their best schedule
    auto p2 = [](double v) { return (int)std::lround(std::log2(std::max(v, 1.0))); };
    char b[96];
    std::snprintf(b, sizeof(b), "fp%d-R2^%d-N2^%d", (int)(8 * sizeof(T)), p2((double)R), p2((double)ntot));
    return std::string(b);
  }

  int counters(int64_t* c, int n) override {
    std::vector<Dyn<T>> h;
    int r = read_dyn(h);
    if (r) return r;
    int64_t status = 0, iters = 0, rebuilds = 0;
    for (const Dyn<T>& y : h) { status |= y.status; iters += (int64_t)y.rattle_iters; rebuilds += (int64_t)y.rebuilds; }
    const int64_t v[6] = {launches, replays, status, iters, rebuilds, cstep};
    for (int k = 0; k < n && k < 6; ++k) c[k] = v[k];
    return MPCMD_OK;
  }

  int event_record(int slot) override {
    if (slot < 0 || slot >= 8) return MPCMD_ERR_CONFIG;
    ECK(cudaEventRecord(ev[slot], st));
    return MPCMD_OK;
  }
  int event_elapsed(int a, int b, double* ms) override {
    if (a < 0 || a >= 8 || b < 0 || b >= 8 || !ms) return MPCMD_ERR_CONFIG;
    ECK(cudaEventSynchronize(ev[b]));
    float f = 0.f;
    ECK(cudaEventElapsedTime(&f, ev[a], ev[b]));
    *ms = f;
    return MPCMD_OK;
  }
  int synchronize() override {
    ECK(cudaStreamSynchronize(st));
    return MPCMD_OK;
  }
};

template <typename T>
EnsembleBase* make_ensemble(const mpcmd_ensemble_config& cfg, const mpcmd_replica* reps, int* status) {
  Ensemble<T>* e = new Ensemble<T>();
  int r = e->create(cfg, reps);
  if (r != MPCMD_OK) {
    delete e;
    *status = r;
    return nullptr;
  }
  *status = MPCMD_OK;
  return e;
}

}  // namespace ens
}  // namespace mpcmd
