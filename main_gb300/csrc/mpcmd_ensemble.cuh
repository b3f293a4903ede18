// Batched ensemble: many independent single-dimer replicas of the plain
// periodic run advanced together on one GPU.
//
// Layout.  All replicas share one structure of arrays: replica r owns the
// particles [poff, poff + n), the cells [coff, coff + ncell) of every per-cell
// table and the shell slots [soff, soff + scap).  A particle is stored as in
// the single-box engine (packed cell + offset in T, velocity in T, species
// flag), so each replica's kernels use the engine's device helpers with the
// replica's own KParams.
//
// Work.  Every kernel is one persistent launch over all replicas: a block
// takes a work tile (a run of consecutive particles, cells or shell entries of
// one replica) at a time, so a block-level reduction is always a reduction
// within one replica.  The particle and cell tiles are fixed at creation; the
// shell tiles follow the shell sizes, which each replica's rebuilds change on
// the device (k_ens_finalize rescans them).  Nothing in a collision period
// needs the host: the rebuild decision of each replica (displacement
// criterion, time_penetrate, collision step: evolve_mod.f95:457-465) is taken
// by k_ens_dimer and read by the rebuild kernel, which skips the tiles of the
// replicas that do not rebuild.
//
// Step sequence (main_pattern.f95:203-225 for every replica), kernels in
// launch order:
//   k_ens_dimer  (VEL)   totals and RATTLE velocities of the previous step
//   k_ens_dimer  (POS)   time_count + 1, RATTLE positions, rebuild decision
//   k_ens_rebuild        lazy streaming of the outside particles and the new
//                        lists of the rebuilding replicas
//   k_ens_finalize       time_penetrate, shell tiles, step counter
//   k_ens_force          forces, catalysis, sphere sums, second half kick; fused
//                        with the next step's first half kick and free flight
//   collision steps:     k_ens_collide (shifted keys, collision sums,
//                        distribute counts), k_ens_cells (centre of mass, axis,
//                        reaction), k_ens_rotate
#pragma once
#include <cooperative_groups.h>
#include <cstdint>
#include <cuda_runtime.h>

#include "mpcmd.h"
#include "mpcmd_kernels.cuh"   // lj, rotate_v and the engine's device helpers

namespace mpcmd {
namespace ens {

namespace cg = cooperative_groups;

constexpr int MAX_BLOCK = 256;
constexpr uint8_t E_IN = 0x20;   // in the list of either sphere at the last rebuild

enum : int { E_ERR_CELL = 1, E_ERR_SHELL = 2, E_ERR_RATTLE = 4, E_ERR_INIT = 8 };
enum : int { M_LAZY = 1, M_LISTS = 2 };          // k_ens_rebuild
enum : int { M_FORCE = 1, M_ADVANCE = 2 };       // k_ens_force
enum : int { M_VEL = 1, M_POS = 2 };             // k_ens_dimer

// Constant per replica.
template <typename T>
struct Rep {
  KParams<T> kp;          // box, species, LJ and collision constants of the replica
  int64_t poff, n;        // particles [poff, poff + n)
  int64_t coff;           // cells [coff, coff + kp.ncell)
  int64_t soff, scap;     // shell slots [soff, soff + scap)
  double skin;
  double mcn;             // Mc + Mn
  double sd[4];           // sqrt(kT / m) per species (initial velocities)
};

// Mutable per replica.
template <typename T>
struct Dyn {
  double dpos[6], dvel[6], dfrc[6], dq[6];   // C then N sphere
  double facc[8];          // per sphere: -sum of the pair forces (xyz) and the pair potential
  double pot;              // potential of the last force evaluation
  SphereRel<T> srel[2];
  double shift[3];         // grid shift of the current collision
  float shf[3];
  int time_count, time_penetrate;
  int rebuild, status;
  unsigned n_shell, pad;
  unsigned long long maxmsd;   // bits (double) of the largest max_solvent_dist of this step
  unsigned long long maxv2;    // bits (double) of the largest v^2 at this step's rebuild
  unsigned long long rattle_iters, rebuilds;
  double vsum[4];          // initial placement: velocity sums for the mean removal
  double vdot_sum;         // propulsion speed samples since the last reset
  long long vdot_n;
};

struct Glob {
  unsigned cstep;          // step being executed (advanced by k_ens_finalize)
  unsigned ntiles_s;       // shell tiles
  int status;
  int pad;
};

template <typename T>
struct EDev {
  const Rep<T>* rep;
  Dyn<T>* dyn;
  Glob* g;
  int R;
  int mpc_every;
  // particles
  uint32_t* cell;
  T *ox, *oy, *oz, *vx, *vy, *vz;
  uint8_t* flag;
  uint32_t* pkey;          // shifted collision cell (collision steps)
  // gather target of the sort
  uint32_t* cell2;
  T *ox2, *oy2, *oz2, *vx2, *vy2, *vz2;
  uint8_t* flag2;
  uint32_t* sidx;
  // shell
  uint32_t* sh_idx;        // particle of each slot
  uint8_t* sh_mask;        // bit 0 in the C list, bit 1 in the N list
  T* sh_fp;                // [slot * 6]: pair force with C (xyz), with N (xyz)
  T* sh_msd;               // max_solvent_dist since the last rebuild
  // cells (replica offsets coff)
  void* acc;               // float4 (FP32) or 4 doubles (FP64): count, sum v
  T* rot;                  // [cell * 6] centre-of-mass velocity and axis
  uint32_t* dcnt;          // packed per-species counts
  uint32_t* dfirst;        // [cell * 4] first-member keys
  uint32_t* order_rank;    // position of each cell in the replica's sort order
  uint32_t *scnt, *sstart, *sfill;
  // work tiles
  const uint32_t* pt_rep;
  const int64_t* pt_lo;
  const int64_t* pt_hi;
  int n_ptiles;
  const uint32_t* ct_rep;
  const int64_t* ct_lo;    // local cell range of the tile
  const int64_t* ct_hi;
  int n_ctiles;
  uint32_t* st_prefix;     // [R + 1] first shell tile of each replica
  uint32_t* rt_prefix;     // [R + 1] first rebuild tile of each replica (0 tiles when it does not rebuild)
  int tile;                // particles per tile
  // samples
  float* axes;             // [R * hist * 3]
  int hist;
  uint32_t* field;         // [R * nz * nr]
  int nz, nr;
  float zmax, rmax;
};

// ------------------------------------------------------------- helpers ----
template <typename T>
__device__ __forceinline__ void acc_add(void* acc, int64_t c, T vx, T vy, T vz);
template <>
__device__ __forceinline__ void acc_add<float>(void* acc, int64_t c, float vx, float vy, float vz) {
  atomicAdd(reinterpret_cast<float4*>(acc) + c, make_float4(1.f, vx, vy, vz));
}
template <>
__device__ __forceinline__ void acc_add<double>(void* acc, int64_t c, double vx, double vy, double vz) {
  double* a = reinterpret_cast<double*>(acc) + 4 * c;
  atomicAdd(a + 0, 1.0);
  atomicAdd(a + 1, vx);
  atomicAdd(a + 2, vy);
  atomicAdd(a + 3, vz);
}

__device__ __forceinline__ double dmi(double d, double L) {
  if (d > 0.5 * L) d -= L;
  else if (d < -0.5 * L) d += L;
  return d;
}

// Sum of v over the block into out (thread 0), for nv values; every thread
// of the block must call it.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* sh /* [NV * 32] */) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sh[k * 32 + w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = 0.;
      for (int i = 0; i < nw; ++i) x += sh[k * 32 + i];
      v[k] = x;
    }
  }
  __syncthreads();
}

template <typename T>
__device__ __forceinline__ T block_max(T v, T* sh /* [32] */) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (lane == 0) sh[w] = v;
  __syncthreads();
  T m = (T)0;
  if (threadIdx.x == 0)
    for (int i = 0; i < nw; ++i) m = fmax(m, sh[i]);
  __syncthreads();
  return m;
}

// FP32 build: the eight per-sphere sums of a block, reduced in FP32 (a
// transposing warp reduction: 9 shuffles for 8 values, lane 4v ends with the
// warp total of value v), then over the warps in shared memory; thread v < 8
// returns the block total of value v widened to FP64 (integer ops only), the
// others 0.  FP64 arithmetic per lane would run at the part's FP64 rate.
__device__ __forceinline__ double block_sum8_f32(const float (&a)[8], float* sh /* [8 * 32] */) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4;
  float b[4], c[2];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float send = h16 ? a[k] : a[k + 4], keep = h16 ? a[k + 4] : a[k];
    b[k] = keep + __shfl_xor_sync(full, send, 16);
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const float send = h8 ? b[k] : b[k + 2], keep = h8 ? b[k + 2] : b[k];
    c[k] = keep + __shfl_xor_sync(full, send, 8);
  }
  float e = (h4 ? c[1] : c[0]) + __shfl_xor_sync(full, h4 ? c[0] : c[1], 4);
  e += __shfl_xor_sync(full, e, 2);
  e += __shfl_xor_sync(full, e, 1);
  if ((lane & 3) == 0) sh[(lane >> 2) * 32 + w] = e;
  __syncthreads();
  double out = 0.;
  if (threadIdx.x < 8) {
    float t = 0.f;
    for (int i = 0; i < nw; ++i) t += sh[threadIdx.x * 32 + i];
    out = widen_f32(t);
  }
  __syncthreads();
  return out;
}

template <typename T>
__device__ __forceinline__ void set_srel(Dyn<T>& y, int i, const double* X) {
  const double fx = floor(X[0]), fy = floor(X[1]), fz = floor(X[2]);
  SphereRel<T> r;
  r.cx = (int)fx; r.cy = (int)fy; r.cz = (int)fz;
  r.ox = (T)(X[0] - fx); r.oy = (T)(X[1] - fy); r.oz = (T)(X[2] - fz);
  y.srel[i] = r;
}

// ------------------------------------------------------- initial state ----
// initial_mod.f95:122-345 with the contract draws of the single-box engine
// (k_init_solvent): rejection of positions inside a sphere cutoff, Box-Muller
// velocities (cos branch) of every particle as species A.
template <typename T>
__global__ void k_ens_init(EDev<T> d) {
  const double pi = 3.141592653589793;
  __shared__ double red[3 * 32];
  for (int t = blockIdx.x; t < d.n_ptiles; t += gridDim.x) {
    const uint32_t r = d.pt_rep[t];
    const Rep<T>& R = d.rep[r];
    const KParams<T>& kp = R.kp;
    Dyn<T>& y = d.dyn[r];
    double s[3] = {0., 0., 0.};
    for (int64_t i = d.pt_lo[t] + threadIdx.x; i < d.pt_hi[t]; i += blockDim.x) {
      const uint32_t li = (uint32_t)(i - R.poff);
      bool ok = false;
      uint32_t cell = 0;
      T ox = 0, oy = 0, oz = 0;
      for (uint32_t at = 0; at < 1000000u && !ok; ++at) {
        double ux, uy, uz, un;
        contract_pair(kp.seed, TAG_INIT_POS, li, at, 0, ux, uy);
        contract_pair(kp.seed, TAG_INIT_POS, li, at, 1, uz, un);
        const double X = kp.Ld[0] * ux, Y = kp.Ld[1] * uy, Z = kp.Ld[2] * uz;
        const int cx = min((int)floor(X), kp.lx - 1), cy = min((int)floor(Y), kp.ly - 1),
                  cz = min((int)floor(Z), kp.lz - 1);
        cell = pack_cell(cx, cy, cz);
        ox = (T)(X - cx); oy = (T)(Y - cy); oz = (T)(Z - cz);
        ok = true;
        for (int q = 0; q < 2 && ok; ++q) {
          const double dx = dmi(X - y.dpos[3 * q], kp.Ld[0]);
          const double dy = dmi(Y - y.dpos[3 * q + 1], kp.Ld[1]);
          const double dz = dmi(Z - y.dpos[3 * q + 2], kp.Ld[2]);
          if (dx * dx + dy * dy + dz * dz < (double)kp.cut2_strict[q]) ok = false;
        }
      }
      if (!ok) atomicOr(&y.status, E_ERR_INIT);
      d.cell[i] = cell;
      d.ox[i] = ox; d.oy[i] = oy; d.oz[i] = oz;
      d.flag[i] = 0;
      T* vv[3] = {d.vx, d.vy, d.vz};
      const double sdv = R.sd[0];
      for (int comp = 0; comp < 3; ++comp) {
        double xx, yy;
        contract_pair(kp.seed, TAG_INIT_VEL, li, (uint32_t)comp, 0, xx, yy);
        yy = 1.0 - yy;
        const double th = 2 * pi * xx, Rr = sqrt(-2 * log(yy));
        const T v = (T)(sdv * (Rr * cos(th)) + 0.0);
        vv[comp][i] = v;
        s[comp] += (double)v;
      }
    }
    block_sum<3>(s, red);
    if (threadIdx.x == 0)
      for (int c = 0; c < 3; ++c) atomicAdd(&y.vsum[c], s[c]);
  }
}

// Removal of each replica's mean velocity (the FP32 build rounds at random
// to the neighbouring floats, as the single-box engine's k_sub_mean does).
template <typename T>
__global__ void k_ens_sub_mean(EDev<T> d) {
  for (int t = blockIdx.x; t < d.n_ptiles; t += gridDim.x) {
    const uint32_t r = d.pt_rep[t];
    const Rep<T>& R = d.rep[r];
    const Dyn<T>& y = d.dyn[r];
    const double inv = 1.0 / (double)R.n;
    const double m[3] = {y.vsum[0] * inv, y.vsum[1] * inv, y.vsum[2] * inv};
    T* vv[3] = {d.vx, d.vy, d.vz};
    for (int64_t i = d.pt_lo[t] + threadIdx.x; i < d.pt_hi[t]; i += blockDim.x) {
      const uint32_t li = (uint32_t)(i - R.poff);
      for (int c = 0; c < 3; ++c) {
        const double w = (double)vv[c][i] - m[c];
        if (sizeof(T) == 8) { vv[c][i] = (T)w; continue; }
        float f = (float)w;
        const double rr = w - (double)f;
        if (rr != 0.0) {
          const float g = nextafterf(f, rr > 0.0 ? INFINITY : -INFINITY);
          double u, unused;
          contract_pair(R.kp.seed, TAG_INIT_VEL, li, (uint32_t)(4 + c), 0, u, unused);
          if (u * ((double)g - (double)f) * (rr > 0.0 ? 1.0 : -1.0) < fabs(rr)) f = g;
        }
        vv[c][i] = (T)f;
      }
    }
  }
}

// Host state of one replica <-> device (as k_upload_pos / k_download of the
// single-box engine, periodic geometry).
template <typename T>
__global__ void k_ens_upload(EDev<T> d, int64_t poff, int64_t n, int lx, int ly, int lz, const double* x,
                             const double* y, const double* z, const double* vx, const double* vy,
                             const double* vz, const int32_t* flag) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += stride) {
    const double X[3] = {x[j], y[j], z[j]};
    const int L[3] = {lx, ly, lz};
    int c[3];
    T o[3];
    for (int q = 0; q < 3; ++q) {
      const double f = floor(X[q]);
      c[q] = (int)f;
      o[q] = (T)(X[q] - f);
      if (o[q] >= (T)1) { o[q] -= (T)1; c[q] += 1; }
      c[q] = wrap_cell(c[q], L[q]);
    }
    const int64_t i = poff + j;
    d.cell[i] = pack_cell(c[0], c[1], c[2]);
    d.ox[i] = o[0]; d.oy[i] = o[1]; d.oz[i] = o[2];
    d.vx[i] = (T)vx[j]; d.vy[i] = (T)vy[j]; d.vz[i] = (T)vz[j];
    d.flag[i] = (uint8_t)(flag[j] & FLAG_SPECIES);
  }
}

template <typename T>
__global__ void k_ens_download(EDev<T> d, int64_t poff, int64_t n, double* x, double* y, double* z,
                               double* vx, double* vy, double* vz, int32_t* flag) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += stride) {
    const int64_t i = poff + j;
    const uint32_t c = d.cell[i];
    x[j] = (double)cell_x(c) + (double)d.ox[i];
    y[j] = (double)cell_y(c) + (double)d.oy[i];
    z[j] = (double)cell_z(c) + (double)d.oz[i];
    vx[j] = (double)d.vx[i]; vy[j] = (double)d.vy[i]; vz[j] = (double)d.vz[i];
    flag[j] = (int32_t)(d.flag[i] & FLAG_SPECIES);
  }
}

// ------------------------------------------------------------- rebuild ----
// evolve_mod.f95:465-564 for the replicas that rebuild at this step: lazy
// streaming of the outside particles over the time_count steps since the
// last rebuild (:473-529), then the lists (neighbour_list_mod.f95:6-184): a
// particle within cutoff + skin of either sphere takes a shell slot (which
// sphere lists hold it: sh_mask) and the E_IN flag, and the largest v^2 of
// each replica is kept for time_penetrate (:554-564).  mode M_LAZY, M_LISTS
// or both (a sort runs between the two halves on sort steps).
// Replica of work tile t of a tile prefix (the largest r with prefix[r] <= t).
__device__ __forceinline__ int tile_rep(const uint32_t* prefix, int R, unsigned t) {
  int lo = 0, hi = R - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (prefix[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Plan of a rebuild: the particle tiles of the replicas whose rebuild flag
// k_ens_dimer set, as a prefix over replicas.  One block.
template <typename T>
__global__ void k_ens_plan(EDev<T> d) {
  __shared__ unsigned part[1024];
  const int nt = blockDim.x;
  const int chunk = (d.R + nt - 1) / nt;
  const int lo = min(d.R, (int)threadIdx.x * chunk), hi = min(d.R, lo + chunk);
  unsigned local = 0;
  for (int r = lo; r < hi; ++r)
    if (d.dyn[r].rebuild) local += (unsigned)((d.rep[r].n + d.tile - 1) / d.tile);
  part[threadIdx.x] = local;
  __syncthreads();
  for (int o = 1; o < nt; o <<= 1) {
    unsigned v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
  for (int r = lo; r < hi; ++r) {
    d.rt_prefix[r] = run;
    if (d.dyn[r].rebuild) run += (unsigned)((d.rep[r].n + d.tile - 1) / d.tile);
  }
  if (threadIdx.x == nt - 1) d.rt_prefix[d.R] = part[nt - 1];
}

template <typename T>
__global__ void __launch_bounds__(MAX_BLOCK) k_ens_rebuild(EDev<T> d, int mode) {
  __shared__ T red[32];
  const unsigned ntiles = d.rt_prefix[d.R];
  for (unsigned t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int r = tile_rep(d.rt_prefix, d.R, t);
    Dyn<T>& y = d.dyn[r];
    const Rep<T>& R = d.rep[r];
    const int64_t tlo = R.poff + (int64_t)(t - d.rt_prefix[r]) * d.tile;
    const int64_t thi = min(tlo + (int64_t)d.tile, R.poff + R.n);
    const KParams<T>& kp = R.kp;
    const int tc = y.time_count;
    const SphereRel<T> sC = y.srel[0], sN = y.srel[1];
    T vmax = (T)0;
    for (int64_t i = tlo + threadIdx.x; i < thi; i += blockDim.x) {
      uint32_t cell = d.cell[i];
      T ox = d.ox[i], oy = d.oy[i], oz = d.oz[i];
      T vx = d.vx[i], vy = d.vy[i], vz = d.vz[i];
      uint8_t f = d.flag[i];
      if ((mode & M_LAZY) && !(f & E_IN) && tc > 0) {
        stream_one(kp, (const uint8_t*)nullptr, cell, ox, oy, oz, vx, vy, vz, f, true, tc);
        d.cell[i] = cell;
        d.ox[i] = ox; d.oy[i] = oy; d.oz[i] = oz;
      }
      if (mode & M_LISTS) {
        T dx, dy, dz;
        const T dC = sep2(kp, cell, ox, oy, oz, sC, dx, dy, dz);
        const T dN = sep2(kp, cell, ox, oy, oz, sN, dx, dy, dz);
        const int mask = (dC <= kp.full2[0] ? 1 : 0) | (dN <= kp.full2[1] ? 2 : 0);
        f = mask ? (uint8_t)(f | E_IN) : (uint8_t)(f & ~E_IN);
        d.flag[i] = f;
        vmax = fmax(vmax, vx * vx + vy * vy + vz * vz);
        if (mask) {
          cg::coalesced_group grp = cg::coalesced_threads();
          unsigned base = 0;
          if (grp.thread_rank() == 0) base = atomicAdd(&y.n_shell, (unsigned)grp.size());
          base = grp.shfl(base, 0);
          const int64_t slot = (int64_t)base + grp.thread_rank();
          if (slot < R.scap) {
            const int64_t e = R.soff + slot;
            d.sh_idx[e] = (uint32_t)i;
            d.sh_mask[e] = (uint8_t)mask;
            for (int q = 0; q < 6; ++q) d.sh_fp[6 * e + q] = (T)0;
            d.sh_msd[e] = (T)0;
          } else {
            atomicOr(&y.status, E_ERR_SHELL);
          }
        }
      }
    }
    if (mode & M_LISTS) {
      const T m = block_max(vmax, red);
      if (threadIdx.x == 0 && m > (T)0) atomicMax(&y.maxv2, ord_bits(to_f64(m)));
    }
  }
}

// After the rebuild: time_penetrate of the rebuilt replicas
// (main_pattern.f95:187, evolve_mod.f95:555-563), the shell work tiles of
// every replica, and the step counter.  One block.
template <typename T>
__global__ void k_ens_finalize(EDev<T> d, int shell_block, int advance_step) {
  __shared__ unsigned part[1024];
  const int nt = blockDim.x;
  const int chunk = (d.R + nt - 1) / nt;
  const int lo = min(d.R, (int)threadIdx.x * chunk), hi = min(d.R, lo + chunk);
  unsigned local = 0;
  for (int r = lo; r < hi; ++r) {
    Dyn<T>& y = d.dyn[r];
    const Rep<T>& R = d.rep[r];
    if (y.rebuild) {
      const double maxt = __longlong_as_double((long long)y.maxv2);
      y.time_penetrate = (int)floor((0.5 * R.skin / sqrt(maxt)) / R.kp.dtd);
      y.time_count = 0;
      y.rebuild = 0;
      y.maxv2 = 0ull;
      y.rebuilds += 1;
      if (y.n_shell > (unsigned)R.scap) y.n_shell = (unsigned)R.scap;
    }
    local += (y.n_shell + shell_block - 1) / shell_block;
  }
  part[threadIdx.x] = local;
  __syncthreads();
  // inclusive scan of the per-thread tile counts (Hillis-Steele)
  for (int o = 1; o < nt; o <<= 1) {
    unsigned v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
  for (int r = lo; r < hi; ++r) {
    d.st_prefix[r] = run;
    run += (d.dyn[r].n_shell + shell_block - 1) / shell_block;
  }
  if (threadIdx.x == nt - 1) {
    d.st_prefix[d.R] = part[nt - 1];
    d.g->ntiles_s = part[nt - 1];
    if (advance_step) d.g->cstep += 1;
  }
}

// --------------------------------------------------------------- forces ----
// Over the shell of every replica: LJ 12-6 with each listed sphere within its
// cutoff and the catalytic A -> B conversion on the C sphere
// (forces_mod.f95:62-136), the sphere sums (evolve_mod.f95:605-636) and the
// second half kick (:645-670) [M_FORCE]; then the first half kick and the
// free flight of the next step with max_solvent_dist (:225-316, :457-463)
// [M_ADVANCE].  The kicks add the C pair force, then the N pair force
// (kick_lists order); the FP32 build adds their sum.
template <typename T>
__global__ void __launch_bounds__(MAX_BLOCK) k_ens_force(EDev<T> d, int mode) {
  __shared__ double red[8 * 32];
  __shared__ float redf[8 * 32];
  __shared__ T redm[32];
  const unsigned ntiles = d.g->ntiles_s;
  for (unsigned t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int r = tile_rep(d.st_prefix, d.R, t);
    Dyn<T>& y = d.dyn[r];
    const Rep<T>& R = d.rep[r];
    const KParams<T>& kp = R.kp;
    const int64_t j = (int64_t)(t - d.st_prefix[r]) * blockDim.x + threadIdx.x;
    const bool valid = j < (int64_t)y.n_shell;
    T sums[8] = {(T)0, (T)0, (T)0, (T)0, (T)0, (T)0, (T)0, (T)0};
    T msd = (T)0;
    if (valid) {
      const int64_t e = R.soff + j;
      const uint32_t i = d.sh_idx[e];
      const int mask = d.sh_mask[e];
      uint32_t cell = d.cell[i];
      T ox = d.ox[i], oy = d.oy[i], oz = d.oz[i];
      T vx = d.vx[i], vy = d.vy[i], vz = d.vz[i];
      uint8_t f = d.flag[i];
      T fp[6];
      for (int q = 0; q < 6; ++q) fp[q] = d.sh_fp[6 * e + q];
      if (mode & M_FORCE) {
        for (int s = 0; s < 2; ++s) {
          fp[3 * s] = fp[3 * s + 1] = fp[3 * s + 2] = (T)0;
          if (!(mask & (1 << s))) continue;
          T dx, dy, dz;
          const T dR2 = sep2(kp, cell, ox, oy, oz, y.srel[s], dx, dy, dz);
          if (dR2 <= kp.cut2[s]) {
            int sp = f & FLAG_SPECIES;
            if (s == 0 && sp == 0) { sp = 1; f = (uint8_t)((f & ~FLAG_SPECIES) | 1); }
            const T E = s == 0 ? kp.eps_c[sp] : kp.eps_n[sp];
            T fx, fy, fz, u;
            lj(kp, s, E, dR2, dx, dy, dz, fx, fy, fz, u);
            fp[3 * s] = fx; fp[3 * s + 1] = fy; fp[3 * s + 2] = fz;
            sums[4 * s + 0] -= fx; sums[4 * s + 1] -= fy;
            sums[4 * s + 2] -= fz; sums[4 * s + 3] += u;
          }
        }
      }
      const T h = kp.hIM[f & FLAG_SPECIES];
      const int nk = ((mode & M_FORCE) ? 1 : 0) + ((mode & M_ADVANCE) ? 1 : 0);
      for (int k = 0; k < nk; ++k) {
        if (sizeof(T) == 8) {
          vx = vx + h * fp[0]; vy = vy + h * fp[1]; vz = vz + h * fp[2];
          vx = vx + h * fp[3]; vy = vy + h * fp[4]; vz = vz + h * fp[5];
        } else {
          vx += h * (fp[0] + fp[3]); vy += h * (fp[1] + fp[4]); vz += h * (fp[2] + fp[5]);
        }
      }
      if (mode & M_ADVANCE) {
        stream_one(kp, (const uint8_t*)nullptr, cell, ox, oy, oz, vx, vy, vz, f, false, 0);
        msd = d.sh_msd[e] + (vx * vx + vy * vy + vz * vz) * (kp.dt * kp.dt);
        d.sh_msd[e] = msd;
        d.cell[i] = cell;
        d.ox[i] = ox; d.oy[i] = oy; d.oz[i] = oz;
      }
      d.vx[i] = vx; d.vy[i] = vy; d.vz[i] = vz;
      d.flag[i] = f;
      if (mode & M_FORCE)
        for (int q = 0; q < 6; ++q) d.sh_fp[6 * e + q] = fp[q];
    }
    if (mode & M_FORCE) {
      if (sizeof(T) == 4) {
        float sf[8];
        for (int q = 0; q < 8; ++q) sf[q] = (float)sums[q];
        const double v = block_sum8_f32(sf, redf);
        if (threadIdx.x < 8 && v != 0.) atomicAdd(&y.facc[threadIdx.x], v);
      } else {
        double sd[8];
        for (int q = 0; q < 8; ++q) sd[q] = (double)sums[q];
        block_sum<8>(sd, red);
        if (threadIdx.x == 0)
          for (int q = 0; q < 8; ++q)
            if (sd[q] != 0.) atomicAdd(&y.facc[q], sd[q]);
      }
    }
    if (mode & M_ADVANCE) {
      const T m = block_max(msd, redm);
      if (threadIdx.x == 0 && m > (T)0) atomicMax(&y.maxmsd, ord_bits(to_f64(m)));
    }
  }
}

// ---------------------------------------------------------------- dimer ----
// One thread per replica, the FP64 operation sequence of the reference:
// M_VEL  sphere totals (evolve_mod.f95:605-636) and RATTLE velocities
//        (:679-724); on a collision step also the propulsion-speed sample
//        (Output_SelkovDimer.f90:168-172) and the grid shift of the collision
//        (mpc_rotation_mod.f95:102-107);
// M_POS  time_count + 1, RATTLE positions of the next step (:320-417) and the
//        rebuild decision (:457-465).
template <typename T>
__global__ void k_ens_dimer(EDev<T> d, int mode, int rattle_max) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= d.R) return;
  Dyn<T>& y = d.dyn[r];
  const Rep<T>& R = d.rep[r];
  const KParams<T>& kp = R.kp;
  const double dt = kp.dtd, Mc = kp.mc, Mn = kp.mn, Dcn = kp.dcn;
  const double hIMc = kp.hIMc, hIMn = kp.hIMn, IIM = kp.IIM;
  // the FP32 build multiplies by precomputed reciprocals and wraps the
  // positions once after the iterations (the constraint uses minimum-image
  // separations); the FP64 build keeps the reference's operation sequence
  constexpr bool fast = sizeof(T) == 4;
  double X1[3], X2[3], V1[3], V2[3], F1[3], F2[3], Q1[3], Q2[3];
  for (int c = 0; c < 3; ++c) {
    X1[c] = y.dpos[c]; X2[c] = y.dpos[3 + c];
    V1[c] = y.dvel[c]; V2[c] = y.dvel[3 + c];
    F1[c] = y.dfrc[c]; F2[c] = y.dfrc[3 + c];
    Q1[c] = y.dq[c]; Q2[c] = y.dq[3 + c];
  }
  unsigned long long iters = 0;
  if (mode & M_VEL) {
    for (int c = 0; c < 3; ++c) { F1[c] = y.facc[c]; F2[c] = y.facc[4 + c]; }
    y.pot = y.facc[3] + y.facc[7];
    for (int q = 0; q < 8; ++q) y.facc[q] = 0.;
    for (int c = 0; c < 3; ++c) { V1[c] = Q1[c] + hIMc * F1[c]; V2[c] = Q2[c] + hIMn * F2[c]; }
    int acc = 0;
    for (;;) {
      double dV[3], dd[3];
      for (int c = 0; c < 3; ++c) { dV[c] = V1[c] - V2[c]; dd[c] = dmi(X1[c] - X2[c], kp.Ld[c]); }
      const double Con2diff = 2.0 * (dV[0] * dd[0] + dV[1] * dd[1] + dV[2] * dd[2]);
      if (fabs(Con2diff) < 1.e-8) break;
      if (acc == rattle_max) { atomicOr(&y.status, E_ERR_RATTLE); break; }
      if (fast) {
        const double O2 = -(0.5 * (IIM * Con2diff) * kp.iD2);
        for (int c = 0; c < 3; ++c) {
          V1[c] = V1[c] + O2 * dd[c] * kp.iMc;
          V2[c] = V2[c] - O2 * dd[c] * kp.iMn;
        }
      } else {
        const double O = -(0.25 * (IIM * Con2diff) / (Dcn * Dcn));
        for (int c = 0; c < 3; ++c) {
          V1[c] = V1[c] + 2.0 * O * dd[c] / Mc;
          V2[c] = V2[c] - 2.0 * O * dd[c] / Mn;
        }
      }
      acc++;
    }
    iters += acc;
    for (int c = 0; c < 3; ++c) {
      y.dvel[c] = V1[c]; y.dvel[3 + c] = V2[c];
      y.dfrc[c] = F1[c]; y.dfrc[3 + c] = F2[c];
    }
    const unsigned step = d.g->cstep;
    if (step % (unsigned)d.mpc_every == 0u) {
      double dd[3], len2 = 0.;
      for (int c = 0; c < 3; ++c) { dd[c] = dmi(X1[c] - X2[c], kp.Ld[c]); len2 += dd[c] * dd[c]; }
      const double len = sqrt(len2);
      double s = 0.;
      for (int c = 0; c < 3; ++c) s += ((Mc * V1[c] + Mn * V2[c]) / (Mn + Mc)) * (dd[c] / len);
      if (d.hist > 0) {
        const long long k = y.vdot_n;
        if (k < d.hist)
          for (int c = 0; c < 3; ++c) d.axes[((size_t)r * d.hist + k) * 3 + c] = (float)(dd[c] / len);
      }
      y.vdot_sum += s;
      y.vdot_n += 1;
      double u0, u1, u2, u3;
      contract_pair(kp.seed, TAG_SHIFT, 0, 0, step, u0, u1);
      contract_pair(kp.seed, TAG_SHIFT, 0, 1, step, u2, u3);
      y.shift[0] = u0 - 0.5; y.shift[1] = u1 - 0.5; y.shift[2] = u2 - 0.5;
      for (int c = 0; c < 3; ++c) y.shf[c] = (float)y.shift[c];
    }
  }
  if (mode & M_POS) {
    const unsigned step = d.g->cstep + 1u;
    y.time_count += 1;
    double pr1[3], pr2[3], dP[3];
    for (int c = 0; c < 3; ++c) { pr1[c] = X1[c]; pr2[c] = X2[c]; dP[c] = dmi(X1[c] - X2[c], kp.Ld[c]); }
    for (int c = 0; c < 3; ++c) { Q1[c] = V1[c] + hIMc * F1[c]; Q2[c] = V2[c] + hIMn * F2[c]; }
    for (int c = 0; c < 3; ++c) { X1[c] = X1[c] + dt * Q1[c]; X2[c] = X2[c] + dt * Q2[c]; }
    if (!fast)
      for (int c = 0; c < 3; ++c) {
        X1[c] = X1[c] - kp.Ld[c] * floor(X1[c] / kp.Ld[c]);
        X2[c] = X2[c] - kp.Ld[c] * floor(X2[c] / kp.Ld[c]);
      }
    int acc = 0;
    for (;;) {
      double dd[3];
      for (int c = 0; c < 3; ++c) dd[c] = dmi(X1[c] - X2[c], kp.Ld[c]);
      const double Con1diff = (dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]) - Dcn * Dcn;
      if (fabs(Con1diff) < 1.e-6) break;
      if (acc == rattle_max) { atomicOr(&y.status, E_ERR_RATTLE); break; }
      const double den = dd[0] * dP[0] + dd[1] * dP[1] + dd[2] * dP[2];
      if (fast) {
        // the iteration converges to the tolerance whatever the last bits of
        // G are: a float reciprocal refined twice replaces the division
        double rr = (double)__frcp_rn((float)den);
        rr = rr * (2.0 - den * rr);
        rr = rr * (2.0 - den * rr);
        const double G2 = 2.0 * (-(0.25 * Con1diff * IIM) * rr);
        for (int c = 0; c < 3; ++c) {
          X1[c] = pr1[c] + Q1[c] * dt + G2 * dP[c] * kp.iMc;
          X2[c] = pr2[c] + Q2[c] * dt - G2 * dP[c] * kp.iMn;
          Q1[c] = Q1[c] + G2 * dP[c] * kp.iMcdt;
          Q2[c] = Q2[c] - G2 * dP[c] * kp.iMndt;
        }
      } else {
        const double G = -(0.25 * Con1diff * IIM / den);
        for (int c = 0; c < 3; ++c) {
          X1[c] = pr1[c] + Q1[c] * dt + 2.0 * G * dP[c] / Mc;
          X2[c] = pr2[c] + Q2[c] * dt - 2.0 * G * dP[c] / Mn;
        }
        for (int c = 0; c < 3; ++c) {
          X1[c] = X1[c] - kp.Ld[c] * floor(X1[c] / kp.Ld[c]);
          X2[c] = X2[c] - kp.Ld[c] * floor(X2[c] / kp.Ld[c]);
        }
        for (int c = 0; c < 3; ++c) {
          Q1[c] = Q1[c] + 2.0 * G * dP[c] / (Mc * dt);
          Q2[c] = Q2[c] - 2.0 * G * dP[c] / (Mn * dt);
        }
      }
      acc++;
    }
    if (fast)
      for (int c = 0; c < 3; ++c) {
        const double L = kp.Ld[c];
        if (X1[c] >= L) X1[c] -= L; else if (X1[c] < 0.0) X1[c] += L;
        if (X2[c] >= L) X2[c] -= L; else if (X2[c] < 0.0) X2[c] += L;
        if (!(X1[c] >= 0.0 && X1[c] < L)) X1[c] = X1[c] - L * floor(X1[c] / L);
        if (!(X2[c] >= 0.0 && X2[c] < L)) X2[c] = X2[c] - L * floor(X2[c] / L);
      }
    iters += acc;
    for (int c = 0; c < 3; ++c) {
      y.dpos[c] = X1[c]; y.dpos[3 + c] = X2[c];
      y.dq[c] = Q1[c]; y.dq[3 + c] = Q2[c];
    }
    set_srel(y, 0, X1);
    set_srel(y, 1, X2);
    const double maxv = __longlong_as_double((long long)y.maxmsd);
    const double thr = (double)kp.msd_thr;
    const bool rb = maxv > thr || y.time_count == y.time_penetrate || step % (unsigned)d.mpc_every == 0u;
    y.maxmsd = 0ull;
    if (rb) {
      y.rebuild = 1;
      y.n_shell = 0;
      y.maxv2 = 0ull;
    }
  }
  if (iters) y.rattle_iters += iters;
}

// The FP32 build's dimer step with the three Cartesian components of a
// replica's dimer on three lanes of a 4-lane group (the fourth lane holds
// zeros and the replica's scalar work): the update of k_ens_dimer's fast
// path, with every dot product summed over the group.  At GB300's FP64 rate
// the per-replica chain of FP64 instructions sets the kernel's time, and the
// split shortens it about threefold.  The group sums add the same terms in
// the same order as the one-thread form ((x + y) + (z + 0)).
template <typename T>
__global__ void k_ens_dimer_split(EDev<T> d, int mode, int rattle_max) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int r = t >> 2, c = t & 3;
  const unsigned gmask = 0xFu << (threadIdx.x & 28);   // this group's four lanes
  const bool live = r < d.R;                            // the whole group agrees
  Dyn<T>& y = d.dyn[live ? r : 0];
  const Rep<T>& R = d.rep[live ? r : 0];
  const KParams<T>& kp = R.kp;
  const bool comp = c < 3;
  const double L = kp.Ld[comp ? c : 0];
  const double dt = kp.dtd, Mc = kp.mc, Mn = kp.mn, Dcn = kp.dcn;
  const double hIMc = kp.hIMc, hIMn = kp.hIMn, IIM = kp.IIM;
  double X1 = 0., X2 = 0., V1 = 0., V2 = 0., F1 = 0., F2 = 0., Q1 = 0., Q2 = 0.;
  if (live && comp) {
    X1 = y.dpos[c]; X2 = y.dpos[3 + c];
    V1 = y.dvel[c]; V2 = y.dvel[3 + c];
    F1 = y.dfrc[c]; F2 = y.dfrc[3 + c];
    Q1 = y.dq[c]; Q2 = y.dq[3 + c];
  }
  unsigned long long iters = 0;
  if (mode & M_VEL) {
    if (live) {
      // lane c takes the sphere sums c and 4 + c (lane 3: the potentials)
      const double a1 = y.facc[c], a2 = y.facc[4 + c];
      y.facc[c] = 0.; y.facc[4 + c] = 0.;
      if (comp) { F1 = a1; F2 = a2; }
      else y.pot = a1 + a2;
    }
    if (comp) { V1 = Q1 + hIMc * F1; V2 = Q2 + hIMn * F2; }
    int acc = 0;
    for (;;) {
      const double dd = comp ? dmi(X1 - X2, L) : 0.;
      const double Con2diff = 2.0 * group4_sum(gmask, (V1 - V2) * dd);
      if (!live || fabs(Con2diff) < 1.e-8) break;
      if (acc == rattle_max) { if (c == 0) atomicOr(&y.status, E_ERR_RATTLE); break; }
      const double O2 = -(0.5 * (IIM * Con2diff) * kp.iD2);
      V1 = V1 + O2 * dd * kp.iMc;
      V2 = V2 - O2 * dd * kp.iMn;
      acc++;
    }
    iters += acc;
    if (live && comp) {
      y.dvel[c] = V1; y.dvel[3 + c] = V2;
      y.dfrc[c] = F1; y.dfrc[3 + c] = F2;
    }
    const unsigned step = d.g->cstep;
    if (step % (unsigned)d.mpc_every == 0u) {
      const double dd = comp ? dmi(X1 - X2, L) : 0.;
      const double len = sqrt(group4_sum(gmask, dd * dd));
      const double s = group4_sum(gmask, comp ? ((Mc * V1 + Mn * V2) / (Mn + Mc)) * (dd / len) : 0.);
      if (live) {
        const long long k = y.vdot_n;
        if (d.hist > 0 && k < d.hist && comp) d.axes[((size_t)r * d.hist + k) * 3 + c] = (float)(dd / len);
        __syncwarp(gmask);   // every lane has read vdot_n
        if (c == 0) {
          y.vdot_sum += s;
          y.vdot_n = k + 1;
          double u0, u1, u2, u3;
          contract_pair(kp.seed, TAG_SHIFT, 0, 0, step, u0, u1);
          contract_pair(kp.seed, TAG_SHIFT, 0, 1, step, u2, u3);
          y.shift[0] = u0 - 0.5; y.shift[1] = u1 - 0.5; y.shift[2] = u2 - 0.5;
          for (int q = 0; q < 3; ++q) y.shf[q] = (float)y.shift[q];
        }
      }
    }
  }
  if (mode & M_POS) {
    const unsigned step = d.g->cstep + 1u;
    const double pr1 = X1, pr2 = X2;
    const double dP = comp ? dmi(X1 - X2, L) : 0.;
    if (comp) {
      Q1 = V1 + hIMc * F1; Q2 = V2 + hIMn * F2;
      X1 = X1 + dt * Q1; X2 = X2 + dt * Q2;
    }
    int acc = 0;
    for (;;) {
      const double dd = comp ? dmi(X1 - X2, L) : 0.;
      const double Con1diff = group4_sum(gmask, dd * dd) - Dcn * Dcn;
      if (!live || fabs(Con1diff) < 1.e-6) break;
      if (acc == rattle_max) { if (c == 0) atomicOr(&y.status, E_ERR_RATTLE); break; }
      const double den = group4_sum(gmask, dd * dP);
      // a float reciprocal refined twice replaces the division (the
      // iteration converges to the tolerance whatever G's last bits are)
      double rr = (double)__frcp_rn((float)den);
      rr = rr * (2.0 - den * rr);
      rr = rr * (2.0 - den * rr);
      const double G2 = 2.0 * (-(0.25 * Con1diff * IIM) * rr);
      X1 = pr1 + Q1 * dt + G2 * dP * kp.iMc;
      X2 = pr2 + Q2 * dt - G2 * dP * kp.iMn;
      Q1 = Q1 + G2 * dP * kp.iMcdt;
      Q2 = Q2 - G2 * dP * kp.iMndt;
      acc++;
    }
    iters += acc;
    if (live && comp) {
      if (X1 >= L) X1 -= L; else if (X1 < 0.0) X1 += L;
      if (X2 >= L) X2 -= L; else if (X2 < 0.0) X2 += L;
      if (!(X1 >= 0.0 && X1 < L)) X1 = X1 - L * floor(X1 / L);
      if (!(X2 >= 0.0 && X2 < L)) X2 = X2 - L * floor(X2 / L);
      y.dpos[c] = X1; y.dpos[3 + c] = X2;
      y.dq[c] = Q1; y.dq[3 + c] = Q2;
      // the sphere positions as cell + offset (set_srel), one axis per lane
      const double f1 = floor(X1), f2 = floor(X2);
      SphereRel<T>& r1 = y.srel[0];
      SphereRel<T>& r2 = y.srel[1];
      if (c == 0) { r1.cx = (int)f1; r1.ox = (T)(X1 - f1); r2.cx = (int)f2; r2.ox = (T)(X2 - f2); }
      else if (c == 1) { r1.cy = (int)f1; r1.oy = (T)(X1 - f1); r2.cy = (int)f2; r2.oy = (T)(X2 - f2); }
      else { r1.cz = (int)f1; r1.oz = (T)(X1 - f1); r2.cz = (int)f2; r2.oz = (T)(X2 - f2); }
    }
    if (live && c == 3) {
      // the rebuild decision (evolve_mod.f95:457-465)
      const int tc = y.time_count + 1;
      y.time_count = tc;
      const double maxv = __longlong_as_double((long long)y.maxmsd);
      const double thr = (double)kp.msd_thr;
      const bool rb = maxv > thr || tc == y.time_penetrate || step % (unsigned)d.mpc_every == 0u;
      y.maxmsd = 0ull;
      if (rb) {
        y.rebuild = 1;
        y.n_shell = 0;
        y.maxv2 = 0ull;
      }
    }
  }
  if (live && c == 0 && iters) y.rattle_iters += iters;
}

// ------------------------------------------------------------ collision ----
// mpc_rotation_mod.f95:110-160 (shifted cell of every particle, collision
// sums) fused with distribute_mod.f95:95-182 (per-species counts and first
// members on the unshifted cells, skipping the particles inside a sphere
// cutoff; outside-list members order before inside-list members).
template <typename T>
__global__ void __launch_bounds__(MAX_BLOCK) k_ens_collide(EDev<T> d) {
  for (int t = blockIdx.x; t < d.n_ptiles; t += gridDim.x) {
    const uint32_t r = d.pt_rep[t];
    const Rep<T>& R = d.rep[r];
    const KParams<T>& kp = R.kp;
    Dyn<T>& y = d.dyn[r];
    T sx, sy, sz;
    if (sizeof(T) == 4) { sx = (T)y.shf[0]; sy = (T)y.shf[1]; sz = (T)y.shf[2]; }
    else { sx = (T)y.shift[0]; sy = (T)y.shift[1]; sz = (T)y.shift[2]; }
    const SphereRel<T> sC = y.srel[0], sN = y.srel[1];
    const int lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    // every lane of a warp takes part in every iteration (the run
    // aggregation shuffles over the whole warp); lanes past the tile end
    // carry a key of their own and nothing to add
    for (int64_t i0 = d.pt_lo[t]; i0 < d.pt_hi[t]; i0 += blockDim.x) {
      const int64_t i = i0 + threadIdx.x;
      const bool valid = i < d.pt_hi[t];
      uint32_t key = 0xFFFFFFFFu - (uint32_t)lane, cid = 0xFFFFFFFFu - (uint32_t)lane;
      T vx = (T)0, vy = (T)0, vz = (T)0;
      unsigned cadd = 0u;
      if (valid) {
        const uint32_t cell = d.cell[i];
        const T ox = d.ox[i], oy = d.oy[i], oz = d.oz[i];
        const uint8_t f = d.flag[i];
        vx = d.vx[i]; vy = d.vy[i]; vz = d.vz[i];
        key = shifted_key(kp, cell, ox, oy, oz, sx, sy, sz);
        d.pkey[i] = key;
        bool bulk = true;
        if (f & E_IN) {
          T dx, dy, dz;
          if (sep2(kp, cell, ox, oy, oz, sC, dx, dy, dz) <= kp.cut2[0] ||
              sep2(kp, cell, ox, oy, oz, sN, dx, dy, dz) <= kp.cut2[1])
            bulk = false;
        }
        if (bulk) {
          const int sp = f & FLAG_SPECIES;
          cid = unshifted_id(kp.lx, kp.ly, cell);
          cadd = 1u << (8 * sp);
          // only the first B of a cell is ever relabelled (reaction_mod.f95:59)
          if (sp == 1) atomicMin(&d.dfirst[4 * (R.coff + cid) + 1], ((f & E_IN) ? 0x80000000u : 0u) | (uint32_t)i);
        }
      }
      // collision sums: runs of equal shifted keys over adjacent lanes (the
      // particles are in cell order), one atomic per run
      {
        const uint32_t prev = __shfl_up_sync(full, key, 1);   // every lane shuffles
        const unsigned heads = __ballot_sync(full, lane == 0 || prev != key);
        const int start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
        T c = valid ? (T)1 : (T)0;
        for (int o = 1; o < 32; o <<= 1) {
          const T c2 = __shfl_up_sync(full, c, o), x2 = __shfl_up_sync(full, vx, o);
          const T y2 = __shfl_up_sync(full, vy, o), z2 = __shfl_up_sync(full, vz, o);
          if (lane - o >= start) { c += c2; vx += x2; vy += y2; vz += z2; }
        }
        const bool tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
        if (tail && valid) {
          if (sizeof(T) == 4) {
            atomicAdd(reinterpret_cast<float4*>(d.acc) + (R.coff + key), make_float4((float)c, (float)vx, (float)vy, (float)vz));
          } else {
            double* a = reinterpret_cast<double*>(d.acc) + 4 * (R.coff + key);
            atomicAdd(a + 0, (double)c); atomicAdd(a + 1, (double)vx);
            atomicAdd(a + 2, (double)vy); atomicAdd(a + 3, (double)vz);
          }
        }
      }
      // distribute counts: runs of equal unshifted cells, one atomic per run
      {
        const uint32_t prev = __shfl_up_sync(full, cid, 1);
        const unsigned heads = __ballot_sync(full, lane == 0 || prev != cid);
        const int start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
        for (int o = 1; o < 32; o <<= 1) {
          const unsigned a2 = __shfl_up_sync(full, cadd, o);
          if (lane - o >= start) cadd += a2;
        }
        const bool tail = lane == 31 || ((heads >> (lane + 1)) & 1u);
        if (tail && cadd) {
          const unsigned old = atomicAdd(&d.dcnt[R.coff + cid], cadd);
          for (int sp = 0; sp < 4; ++sp)
            if (((old >> (8 * sp)) & 255u) + ((cadd >> (8 * sp)) & 255u) > (unsigned)kp.cell_capacity)
              atomicOr(&y.status, E_ERR_CELL);
        }
      }
    }
  }
}

// mpc_rotation_mod.f95:163-194 (centre of mass and random axis per shifted
// cell) and reaction_mod.f95:41-62 (B -> A on the first B of the cell with
// probability 1 - exp(-k1 nB tau)), one thread per cell; the tables are
// cleared for the next collision.  The FP32 build takes the axis and the
// reaction draw from the leading 32-bit Philox words, with the FP64 draw
// inside the guard band of the decision, as the single-box engine does.
template <typename T>
__global__ void __launch_bounds__(MAX_BLOCK) k_ens_cells(EDev<T> d) {
  const double pi = 3.141592653589793;
  const unsigned step = d.g->cstep;
  for (int t = blockIdx.x; t < d.n_ctiles; t += gridDim.x) {
    const uint32_t r = d.ct_rep[t];
    const Rep<T>& R = d.rep[r];
    const KParams<T>& kp = R.kp;
    for (int64_t lc = d.ct_lo[t] + threadIdx.x; lc < d.ct_hi[t]; lc += blockDim.x) {
      const int64_t c = R.coff + lc;
      T cmx = (T)0, cmy = (T)0, cmz = (T)0;
      if (sizeof(T) == 4) {
        float4* ac = reinterpret_cast<float4*>(d.acc) + c;
        const float4 v = *ac;
        if (v.x != 0.f) { cmx = (T)(v.y / v.x); cmy = (T)(v.z / v.x); cmz = (T)(v.w / v.x); }
        *ac = make_float4(0.f, 0.f, 0.f, 0.f);
      } else {
        double* ac = reinterpret_cast<double*>(d.acc) + 4 * c;
        const double n = ac[0];
        if (n != 0.) { cmx = (T)(ac[1] / n); cmy = (T)(ac[2] / n); cmz = (T)(ac[3] / n); }
        ac[0] = ac[1] = ac[2] = ac[3] = 0.;
      }
      T ux, uy, uz;
      if (sizeof(T) == 4) {
        uint32_t w0, w2;
        contract_words(kp.seed, TAG_AXIS, (uint32_t)lc, 0, step, w0, w2);
        const float two32 = 2.3283064365386963e-10f;
        const float u1 = (float)w0 * two32;
        const float u2 = (float)w2 * two32, v2 = ((float)(~w2) + 1.f) * two32;
        float sp, cp;
        sincospif(2.f * u1, &sp, &cp);
        const float rr = 2.f * sqrtf(u2 * v2);
        ux = (T)(rr * cp); uy = (T)(rr * sp); uz = (T)(u2 - v2);
      } else {
        double u1, u2;
        contract_pair(kp.seed, TAG_AXIS, (uint32_t)lc, 0, step, u1, u2);
        const double phi = 2.0 * pi * u1, theta = 2.0 * u2 - 1.0;
        ux = (T)(sqrt(1.0 - theta * theta) * cos(phi));
        uy = (T)(sqrt(1.0 - theta * theta) * sin(phi));
        uz = (T)theta;
      }
      T* ro = d.rot + 6 * c;
      ro[0] = cmx; ro[1] = cmy; ro[2] = cmz; ro[3] = ux; ro[4] = uy; ro[5] = uz;
      const unsigned cnt = d.dcnt[c];
      uint32_t* fk = d.dfirst + 4 * c;
      const int nB = (cnt >> 8) & 255u;
      if (nB > 0) {
        bool fire = false;
        bool exact = sizeof(T) != 4;
        if (!exact) {
          uint32_t w0, w2;
          contract_words(kp.seed, TAG_RXN, (uint32_t)lc, 0, step, w0, w2);
          const float u0f = (float)w0 * 2.3283064365386963e-10f;
          const float pf = 1.f - expf(-(kp.kf[0] * (float)nB) * kp.tauf);
          const float g = pf - u0f;
          exact = fabsf(g) < 4e-6f || w0 == 0u;
          fire = g >= 0.f;
        }
        if (exact) {
          double u0, u1;
          contract_pair(kp.seed, TAG_RXN, (uint32_t)lc, 0, step, u0, u1);
          const double a1 = kp.k[0] * (double)nB;
          fire = (0. < u0 && u0 <= 1.0 - exp(-a1 * kp.tau));
        }
        if (fire && fk[1] != 0xFFFFFFFFu) {
          const uint32_t i = fk[1] & 0x7FFFFFFFu;
          d.flag[i] = (uint8_t)(d.flag[i] & ~FLAG_SPECIES);
        }
      }
      d.dcnt[c] = 0u;
      *reinterpret_cast<uint4*>(fk) = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
    }
  }
}

// mpc_rotation_mod.f95:205-228: v <- v_cm + R (v - v_cm) about the cell's axis.
template <typename T>
__global__ void __launch_bounds__(MAX_BLOCK) k_ens_rotate(EDev<T> d) {
  for (int t = blockIdx.x; t < d.n_ptiles; t += gridDim.x) {
    const uint32_t r = d.pt_rep[t];
    const Rep<T>& R = d.rep[r];
    for (int64_t i = d.pt_lo[t] + threadIdx.x; i < d.pt_hi[t]; i += blockDim.x) {
      const T* ro = d.rot + 6 * (R.coff + d.pkey[i]);
      T vx = d.vx[i], vy = d.vy[i], vz = d.vz[i];
      rotate_v(R.kp, ro, vx, vy, vz);
      d.vx[i] = vx; d.vy[i] = vy; d.vz[i] = vz;
    }
  }
}

// ----------------------------------------------------------------- sort ----
// sort_hilbert_mod.f95:6-98 per replica: stable counting sort of the
// particles by the rank of their cell in the replica's cell order.  The
// global scan over all replicas' cells places replica r's particles at
// [poff, poff + n) again, because its cells follow those of replica r - 1.
template <typename T>
__global__ void k_ens_sort_count(EDev<T> d) {
  for (int t = blockIdx.x; t < d.n_ptiles; t += gridDim.x) {
    const Rep<T>& R = d.rep[d.pt_rep[t]];
    for (int64_t i = d.pt_lo[t] + threadIdx.x; i < d.pt_hi[t]; i += blockDim.x) {
      const int64_t c = R.coff + unshifted_id(R.kp.lx, R.kp.ly, d.cell[i]);
      atomicAdd(&d.scnt[R.coff + d.order_rank[c]], 1u);
    }
  }
}

template <typename T>
__global__ void k_ens_sort_fill(EDev<T> d) {
  for (int t = blockIdx.x; t < d.n_ptiles; t += gridDim.x) {
    const Rep<T>& R = d.rep[d.pt_rep[t]];
    for (int64_t i = d.pt_lo[t] + threadIdx.x; i < d.pt_hi[t]; i += blockDim.x) {
      const int64_t c = R.coff + unshifted_id(R.kp.lx, R.kp.ly, d.cell[i]);
      const int64_t k = R.coff + d.order_rank[c];
      const uint32_t pos = d.sstart[k] + atomicAdd(&d.sfill[k], 1u);
      d.sidx[pos] = (uint32_t)i;
    }
  }
}

template <typename T>
__global__ void k_ens_sort_segments(EDev<T> d, int64_t ncell) {
  const uint32_t *scnt = d.scnt, *sstart = d.sstart;
  uint32_t* sidx = d.sidx;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < ncell; k += stride) {
    const uint32_t b = sstart[k], n = scnt[k];
    uint32_t* s = sidx + b;
    for (uint32_t i = 1; i < n; ++i) {
      const uint32_t v = s[i];
      int j = (int)i - 1;
      while (j >= 0 && s[j] > v) { s[j + 1] = s[j]; --j; }
      s[j + 1] = v;
    }
  }
}

template <typename T>
__global__ void k_ens_sort_gather(EDev<T> d, int64_t ntot) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < ntot; q += stride) {
    const uint32_t i = d.sidx[q];
    d.cell2[q] = d.cell[i];
    d.ox2[q] = d.ox[i]; d.oy2[q] = d.oy[i]; d.oz2[q] = d.oz[i];
    d.vx2[q] = d.vx[i]; d.vy2[q] = d.vy[i]; d.vz2[q] = d.vz[i];
    d.flag2[q] = d.flag[i];
  }
}

// ----------------------------------------------------------- observables --
// output_mod.f95:681-806 per replica: solvent momentum, kinetic energy and
// species counts (FP64 sums), into out[r * 8 ...].
template <typename T>
__global__ void k_ens_observables(EDev<T> d, const double* mass /* [R * 4] */, double* out) {
  __shared__ double red[8 * 32];
  for (int t = blockIdx.x; t < d.n_ptiles; t += gridDim.x) {
    const uint32_t r = d.pt_rep[t];
    const double* m = mass + 4 * r;
    double s[8] = {0., 0., 0., 0., 0., 0., 0., 0.};
    for (int64_t i = d.pt_lo[t] + threadIdx.x; i < d.pt_hi[t]; i += blockDim.x) {
      const int sp = d.flag[i] & FLAG_SPECIES;
      const double vx = (double)d.vx[i], vy = (double)d.vy[i], vz = (double)d.vz[i];
      s[0] += m[sp] * vx; s[1] += m[sp] * vy; s[2] += m[sp] * vz;
      s[3] += 0.5 * m[sp] * (vx * vx + vy * vy + vz * vz);
      s[4 + sp] += 1.0;
    }
    block_sum<8>(s, red);
    if (threadIdx.x == 0)
      for (int q = 0; q < 8; ++q) atomicAdd(&out[8 * r + q], s[q]);
  }
}

// ------------------------------------------------------------------ field --
// B particles (species code 1) of each replica counted on nz x nr bins of the
// axial coordinate z in [-zmax, zmax) and the distance r in [0, rmax) from the
// axis through the dimer midpoint along the unit vector C - N.
template <typename T>
__global__ void k_ens_field(EDev<T> d) {
  for (int t = blockIdx.x; t < d.n_ptiles; t += gridDim.x) {
    const uint32_t r = d.pt_rep[t];
    const Rep<T>& R = d.rep[r];
    const Dyn<T>& y = d.dyn[r];
    double dd[3], mid[3], len2 = 0.;
    for (int c = 0; c < 3; ++c) {
      dd[c] = dmi(y.dpos[c] - y.dpos[3 + c], R.kp.Ld[c]);
      len2 += dd[c] * dd[c];
      mid[c] = y.dpos[3 + c] + 0.5 * dd[c];
    }
    const double il = 1.0 / sqrt(len2);
    const float ax = (float)(dd[0] * il), ay = (float)(dd[1] * il), az = (float)(dd[2] * il);
    const float L[3] = {(float)R.kp.Ld[0], (float)R.kp.Ld[1], (float)R.kp.Ld[2]};
    const float fz = (float)d.nz / (2.f * d.zmax), fr = (float)d.nr / d.rmax;
    uint32_t* out = d.field + (size_t)r * d.nz * d.nr;
    for (int64_t i = d.pt_lo[t] + threadIdx.x; i < d.pt_hi[t]; i += blockDim.x) {
      if ((d.flag[i] & FLAG_SPECIES) != 1) continue;
      const uint32_t c = d.cell[i];
      float p[3] = {(float)((double)cell_x(c) - mid[0]) + (float)d.ox[i],
                    (float)((double)cell_y(c) - mid[1]) + (float)d.oy[i],
                    (float)((double)cell_z(c) - mid[2]) + (float)d.oz[i]};
      for (int q = 0; q < 3; ++q) {
        if (p[q] > 0.5f * L[q]) p[q] -= L[q];
        else if (p[q] < -0.5f * L[q]) p[q] += L[q];
      }
      const float z = p[0] * ax + p[1] * ay + p[2] * az;
      const float rx = p[0] - z * ax, ry = p[1] - z * ay, rz = p[2] - z * az;
      const float rr = sqrtf(rx * rx + ry * ry + rz * rz);
      const int iz = (int)floorf((z + d.zmax) * fz), ir = (int)floorf(rr * fr);
      if (iz >= 0 && iz < d.nz && ir >= 0 && ir < d.nr) atomicAdd(&out[iz * d.nr + ir], 1u);
    }
  }
}

}  // namespace ens
}  // namespace mpcmd
