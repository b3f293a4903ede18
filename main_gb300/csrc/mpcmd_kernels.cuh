// Kernels of the mpcmd engine.  Every kernel is templated on the working
// precision T (float for production runs, double for the FP64 parity build)
// and cites the reference loop it replaces.  Included once per precision by
// mpcmd_kernels_f32.cu and mpcmd_kernels_f64.cu.
#pragma once
#include <cooperative_groups.h>
#include <cstdio>
#include "mpcmd_engine.cuh"

namespace cg = cooperative_groups;

namespace mpcmd {

#ifdef MPCMD_CHECKED
#define LAUNCH_COUNT() (++g_kernel_launches, debug_sync(st, __func__, __LINE__))
#else
#define LAUNCH_COUNT() (++g_kernel_launches)
#endif

// ------------------------------------------------------------ helpers ----
template <typename T>
__device__ __forceinline__ void accum_coll(void* acc, uint32_t key, T vx, T vy, T vz);
template <>
__device__ __forceinline__ void accum_coll<float>(void* acc, uint32_t key, float vx, float vy, float vz) {
  atomicAdd(reinterpret_cast<float4*>(acc) + key, make_float4(1.f, vx, vy, vz));
}
template <>
__device__ __forceinline__ void accum_coll<double>(void* acc, uint32_t key, double vx, double vy, double vz) {
  double* a = reinterpret_cast<double*>(acc) + 4 * (size_t)key;
  atomicAdd(a + 0, 1.0);
  atomicAdd(a + 1, vx);
  atomicAdd(a + 2, vy);
  atomicAdd(a + 3, vz);
}

// distribute_mod.f95:95-182: count one particle of species sp in unshifted
// cell cid and keep the smallest ordering key (first member of the list).
template <typename T>
__device__ __forceinline__ void accum_dist(const Dev<T>& d, const KParams<T>& kp, uint32_t cid, int sp,
                                           uint32_t key) {
  unsigned int old = atomicAdd(&d.dcnt[cid], 1u << (8 * sp));
  unsigned int before = (old >> (8 * sp)) & 255u;
  if (before + 1u > (unsigned)kp.cell_capacity) atomicOr(&d.ctr->status, DEV_ERR_CELL_OVERFLOW);
  atomicMin(&d.dfirst[4 * (size_t)cid + sp], key);
}

// Main index of the particle in slot i (slot = index until an order-only
// re-sort moves particles).
template <typename T>
__device__ __forceinline__ uint32_t lid_of(const Dev<T>& d, uint32_t i) {
  return d.lid ? d.lid[i] : i;
}

// Ordering key of a species-list member: group (0 outside, 1 inside when the
// lists put the inside particles last) above the main index (< 2^31).  The
// smallest key of a cell is its first member; 0xFFFFFFFF is "none".
__device__ __forceinline__ uint32_t dist_key(int group, uint32_t idx) {
  return ((uint32_t)group << 31) | idx;
}

// Append i to a list with one atomic per converged group of lanes.
__device__ __forceinline__ void watch_append(unsigned int* counter, uint32_t* list, uint32_t i) {
  cg::coalesced_group g = cg::coalesced_threads();
  unsigned int base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(counter, g.size());
  base = g.shfl(base, 0);
  list[base + g.thread_rank()] = i;
}

// Per-warp staging of list appends in shared memory.  All lanes of a
// converged warp call wl_add once per iteration; the lanes with `pred` set
// are added to the warp's buffer, which goes to the global list with one
// atomic when it is nearly full and at the end (wl_flush).  One atomic per
// WL_CAP entries instead of one per warp iteration keeps a list with
// millions of appends off a single contended counter.
constexpr int WL_CAP = 448;

__device__ __forceinline__ void wl_flush(uint32_t* buf, unsigned& n, unsigned int* gcount, uint32_t* glist) {
  const int lane = threadIdx.x & 31;
  unsigned base = 0;
  if (lane == 0 && n) base = atomicAdd(gcount, n);
  base = __shfl_sync(0xffffffffu, base, 0);
  for (unsigned j = lane; j < n; j += 32) glist[base + j] = buf[j];
  __syncwarp();
  n = 0;
}

__device__ __forceinline__ void wl_add(uint32_t* buf, unsigned& n, bool pred, uint32_t v, unsigned int* gcount,
                                       uint32_t* glist) {
  const unsigned m = __ballot_sync(0xffffffffu, pred);
  const int lane = threadIdx.x & 31;
  if (pred) buf[n + __popc(m & ((1u << lane) - 1u))] = v;
  n += __popc(m);
  __syncwarp();
  if (n > (unsigned)(WL_CAP - 32)) wl_flush(buf, n, gcount, glist);
}

// Block maximum of a non-negative value, folded into the double bits at
// target.  The reduction runs in T; only the block's result is widened (FP64
// instructions are slow on this part).
template <typename T>
__device__ __forceinline__ void block_max_to(unsigned long long* target, T v) {
  __shared__ T red[TPB / 32];
  T m = v;
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    T b = red[0];
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) b = fmax(b, red[i]);
    if (b > (T)0) atomicMax(target, ord_bits(to_f64(b)));
  }
}

// Grid shift of the step in T (the host rounds it to float once).
template <typename T>
__device__ __forceinline__ T step_shift(const StepArgs& a, int c);
template <>
__device__ __forceinline__ float step_shift<float>(const StepArgs& a, int c) { return a.shf[c]; }
template <>
__device__ __forceinline__ double step_shift<double>(const StepArgs& a, int c) { return a.shift[c]; }

// Sum of (fx, fy, fz, u) over the lanes of a converged warp that hold the same
// sphere s (s < 0: nothing), added once per distinct sphere to facc[4s..4s+3].
template <typename T>
__device__ __forceinline__ void warp_sphere_add(double* facc, int s, T fx, T fy, T fz, T u) {
  const unsigned full = 0xffffffffu;
  unsigned remaining = __ballot_sync(full, s >= 0);
  const int lane = threadIdx.x & 31;
  while (remaining) {
    const int src = __ffs(remaining) - 1;
    const int sr = __shfl_sync(full, s, src);
    const unsigned grp = __ballot_sync(full, s == sr);
    const T a0 = s == sr ? fx : (T)0, a1 = s == sr ? fy : (T)0, a2 = s == sr ? fz : (T)0, a3 = s == sr ? u : (T)0;
    // transposing reduction: the first two levels halve the values a lane
    // carries (6 shuffles for the four sums instead of 20); lane 8v ends with
    // the warp total of value v
    const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0;
    T k0 = h16 ? a2 : a0, k1 = h16 ? a3 : a1;
    k0 += __shfl_xor_sync(full, h16 ? a0 : a2, 16);
    k1 += __shfl_xor_sync(full, h16 ? a1 : a3, 16);
    T k = h8 ? k1 : k0;
    k += __shfl_xor_sync(full, h8 ? k0 : k1, 8);
    k += __shfl_xor_sync(full, k, 4);
    k += __shfl_xor_sync(full, k, 2);
    k += __shfl_xor_sync(full, k, 1);
    if ((lane & 7) == 0) atomicAdd(&facc[4 * sr + (lane >> 3)], to_f64(k));
    remaining &= ~grp;
  }
}

// LJ 12-6 cut and shifted (forces_mod.f95:82-92).
template <typename T>
__device__ __forceinline__ void lj(const KParams<T>& kp, int t, T E, T dRsq, T dx, T dy, T dz,
                                   T& fx, T& fy, T& fz, T& u) {
  T IdRsq = (T)1 / dRsq;
  T IdR6 = IdRsq * IdRsq * IdRsq;
  T IdR8 = IdR6 * IdRsq;
  T IdR12 = IdR6 * IdR6;
  T IdR14 = IdR12 * IdRsq;
  T Fbrack = (T)4 * (kp.r12R12[t] * IdR14 - kp.r6R6[t] * IdR8);
  T Ubrack = (T)4 * (kp.R12[t] * IdR12 - kp.R6[t] * IdR6) + (T)1;
  fx = E * Fbrack * dx;
  fy = E * Fbrack * dy;
  fz = E * Fbrack * dz;
  u = E * Ubrack;
}

// A cell's rotation record (centre-of-mass velocity, then axis) is six T at a
// stride of six T, so each pair of values is aligned to twice its size: three
// 8-byte (16-byte in FP64) loads read a record (six scalar loads made
// k_rotate_main 10 % slower).
template <typename T> struct Pair2;
template <> struct Pair2<float> { using type = float2; };
template <> struct Pair2<double> { using type = double2; };

template <typename T>
__device__ __forceinline__ void load_rot(const T* rot, uint32_t key, T* t) {
  using V = typename Pair2<T>::type;
  const V* r = reinterpret_cast<const V*>(rot + 6 * (size_t)key);
  const V a = r[0], b = r[1], c = r[2];
  t[0] = a.x; t[1] = a.y; t[2] = b.x; t[3] = b.y; t[4] = c.x; t[5] = c.y;
}

// Collision rotation of v - v_cm (mpc_rotation_mod.f95:205-228 Rodrigues form;
// RMPC_SelkovDimer.f90:86-118 projection form).
template <typename T>
__device__ __forceinline__ void rotate_v(const KParams<T>& kp, const T* r, T& vx, T& vy, T& vz) {
  const T cmx = r[0], cmy = r[1], cmz = r[2], ux = r[3], uy = r[4], uz = r[5];
  const T c = kp.cosrot, s = kp.sinrot;
  T dx = vx - cmx, dy = vy - cmy, dz = vz - cmz;
  T rx, ry, rz;
  if (kp.rotation_sense > 0) {
    rx = dx * (c + ux * ux * ((T)1 - c)) + dy * (ux * uy * ((T)1 - c) - uz * s) + dz * (ux * uz * ((T)1 - c) + uy * s);
    ry = dx * (ux * uy * ((T)1 - c) + uz * s) + dy * (c + uy * uy * ((T)1 - c)) + dz * (uy * uz * ((T)1 - c) - ux * s);
    rz = dx * (ux * uz * ((T)1 - c) - uy * s) + dy * (uy * uz * ((T)1 - c) + ux * s) + dz * (c + uz * uz * ((T)1 - c));
  } else {
    T P = dx * ux + dy * uy + dz * uz;
    T px = P * ux, py = P * uy, pz = P * uz;
    T qx = dx - px, qy = dy - py, qz = dz - pz;
    T wx = (qy * uz) - (qz * uy), wy = (qz * ux) - (qx * uz), wz = (qx * uy) - (qy * ux);
    rx = px + qx * c + wx * s;
    ry = py + qy * c + wy * s;
    rz = pz + qz * c + wz * s;
  }
  vx = cmx + rx;
  vy = cmy + ry;
  vz = cmz + rz;
}

// ------------------------------------------------------- upload/download --
template <typename T>
__global__ void k_upload_pos(Particles<T> p, KParams<T> kp, const double* v, int comp) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) {
    double x = v[i];
    int L = comp == 0 ? kp.lx : (comp == 1 ? kp.ly : kp.lz);
    double f = floor(x);
    int c = (int)f;
    T o = (T)(x - f);
    if (o >= (T)1) { o -= (T)1; c += 1; }
    if (comp < 2 || kp.geometry == 1) {
      c = wrap_cell(c, L);
    } else {
      if (c >= L) { c = L - 1; o = (T)1; }
      if (c < 0) { c = 0; o = (T)0; }
    }
    uint32_t cell = comp == 0 ? 0u : p.cell[i];
    int cx = comp == 0 ? c : cell_x(cell), cy = comp == 1 ? c : cell_y(cell), cz = comp == 2 ? c : cell_z(cell);
    if (comp == 0) { cy = 0; cz = 0; }
    p.cell[i] = pack_cell(cx, cy, cz);
    (comp == 0 ? p.ox : comp == 1 ? p.oy : p.oz)[i] = o;
  }
}

template <typename T>
__global__ void k_upload_vel(Particles<T> p, KParams<T> kp, const double* v, int comp) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  T* dst = comp == 0 ? p.vx : comp == 1 ? p.vy : p.vz;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) dst[i] = (T)v[i];
}

template <typename T>
__global__ void k_upload_flag(Particles<T> p, KParams<T> kp, const int32_t* f) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride)
    p.flag[i] = (uint8_t)(f[i] & FLAG_SPECIES);
}

template <typename T>
void Launch<T>::upload_comp(const Dev<T>& d, const KParams<T>& kp, const double* src, int comp, cudaStream_t st) {
  const int g = 1024;
  if (comp < 3) k_upload_pos<T><<<g, TPB, 0, st>>>(d.p, kp, src, comp);
  else k_upload_vel<T><<<g, TPB, 0, st>>>(d.p, kp, src, comp - 3);
  LAUNCH_COUNT();
}

template <typename T>
void Launch<T>::upload_flag(const Dev<T>& d, const KParams<T>& kp, const int32_t* src, cudaStream_t st) {
  k_upload_flag<T><<<1024, TPB, 0, st>>>(d.p, kp, src);
  LAUNCH_COUNT();
}

// Host view of one component, as the reference holds it: inside-list
// members at the current step, outside particles at the last rebuild (lazy
// streaming).  A free-flight member (FLAG_PASSIVE) is streamed by the tc steps
// since the last rebuild; a deferred outside state (written at the last full
// pass) by the tc_defer steps from that pass to the last rebuild.
// State of a component as the reference holds it (outside particles at the
// last rebuild: passive members streamed by tc, deferred ones by tc_defer),
// or with `current` every particle at the current step (outside particles
// written at the last rebuild streamed by tc, deferred ones by tc_defer + tc).
template <typename T>
__global__ void k_download(Particles<T> p, const uint32_t* lid, KParams<T> kp, const uint8_t* react_box, double* out,
                           int comp, int tc, int tc_defer, int current) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) {
    uint32_t c = p.cell[i];
    T ox = p.ox[i], oy = p.oy[i], oz = p.oz[i];
    T vx = p.vx[i], vy = p.vy[i], vz = p.vz[i];
    const uint8_t f = p.flag[i];
    int lag = 0;
    if (f & FLAG_PASSIVE) lag = tc;
    else if (!(f & (FLAG_INLIST | FLAG_FRESH | FLAG_HOME_SHELL))) lag = current ? tc_defer + tc : tc_defer;
    else if (current && !(f & (FLAG_INLIST | FLAG_HOME_SHELL))) lag = tc;
    if (lag > 0) {
      uint8_t ff = f;
      stream_one(kp, react_box, c, ox, oy, oz, vx, vy, vz, ff, true, lag);
    }
    double v;
    if (comp == 0) v = (double)cell_x(c) + (double)ox;
    else if (comp == 1) v = (double)cell_y(c) + (double)oy;
    else if (comp == 2) v = (double)cell_z(c) + (double)oz;
    else v = (double)(comp == 3 ? vx : comp == 4 ? vy : vz);
    out[lid ? lid[i] : i] = v;
  }
}

template <typename T>
void Launch<T>::download_convert(const Dev<T>& d, const KParams<T>& kp, double* out, int comp, int tc,
                                 int tc_defer, int current, cudaStream_t st) {
  k_download<T><<<1024, TPB, 0, st>>>(d.p, d.lid, kp, d.react_box, out, comp, tc, tc_defer, current);
  LAUNCH_COUNT();
}

// Concentration fields (output_mod.f95:482-575) on the host view of the
// positions (the k_download reconstruction): counts of species 0 and 1 per
// bin of the three slabs, and the box totals (one atomic per block).
__device__ __forceinline__ int conc_bin(double u, double w, int nb) {
  int j = (int)ceil(u / w);
  j = j < 1 ? 1 : (j > nb ? nb : j);
  return j - 1;
}

template <typename T>
__global__ void k_concentration(Particles<T> p, KParams<T> kp, const uint8_t* react_box, int tc, int tc_defer,
                                ConcArgs c) {
  __shared__ unsigned int blk[2];
  if (threadIdx.x < 2) blk[threadIdx.x] = 0u;
  __syncthreads();
  unsigned int na = 0u, nb = 0u;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) {
    const uint8_t f = p.flag[i];
    const int sp = f & FLAG_SPECIES;
    if (sp > 1) continue;
    uint32_t cl = p.cell[i];
    T ox = p.ox[i], oy = p.oy[i], oz = p.oz[i];
    int lag = 0;
    if (f & FLAG_PASSIVE) lag = tc;
    else if (!(f & (FLAG_INLIST | FLAG_FRESH | FLAG_HOME_SHELL))) lag = tc_defer;
    if (lag > 0) {
      T vx = p.vx[i], vy = p.vy[i], vz = p.vz[i];
      uint8_t ff = f;
      stream_one(kp, react_box, cl, ox, oy, oz, vx, vy, vz, ff, true, lag);
    }
    const double x = (double)cell_x(cl) + (double)ox;
    const double y = (double)cell_y(cl) + (double)oy;
    const double z = (double)cell_z(cl) + (double)oz;
    if (sp == 0) ++na; else ++nb;
    if (z <= c.zs + c.hw && z >= c.zs - c.hw) {
      const int j = conc_bin(x, c.xw, c.nx), k = conc_bin(y, c.yw, c.ny);
      atomicAdd(sp == 0 ? &c.c1a[j] : &c.c1b[j], 1u);
      atomicAdd(sp == 0 ? &c.xya[j + (size_t)c.nx * k] : &c.xyb[j + (size_t)c.nx * k], 1u);
    }
    if (y <= c.ys + c.hw && y >= c.ys - c.hw) {
      const int j = conc_bin(x, c.xw, c.nx), k = conc_bin(z, c.zw, c.nz);
      atomicAdd(sp == 0 ? &c.xza[j + (size_t)c.nx * k] : &c.xzb[j + (size_t)c.nx * k], 1u);
    }
    if (x <= c.xs + c.hw && x >= c.xs - c.hw) {
      const int j = conc_bin(y, c.yw, c.ny), k = conc_bin(z, c.zw, c.nz);
      atomicAdd(sp == 0 ? &c.yza[j + (size_t)c.ny * k] : &c.yzb[j + (size_t)c.ny * k], 1u);
    }
  }
  atomicAdd(&blk[0], na);
  atomicAdd(&blk[1], nb);
  __syncthreads();
  if (threadIdx.x < 2) atomicAdd(&c.tot[threadIdx.x], (unsigned long long)blk[threadIdx.x]);
}

template <typename T>
void Launch<T>::concentration(const Dev<T>& d, const KParams<T>& kp, int tc, int tc_defer, const ConcArgs& c,
                              cudaStream_t st) {
  k_concentration<T><<<1024, TPB, 0, st>>>(d.p, kp, d.react_box, tc, tc_defer, c);
  LAUNCH_COUNT();
}

// Species of every particle.  In the reference's view (outside particles at
// the last rebuild) these are the stored species: a lagging particle of that
// view cannot reach a wall before its lag ends.  With `current` the outside
// particles written at the last rebuild are streamed over the lag as in
// k_download, so a reactive-floor hit in that time (reactive_grid_mod.f95:
// 103-151) changes the species it reports.
template <typename T>
__global__ void k_download_flag(Particles<T> p, const uint32_t* lid, KParams<T> kp, const uint8_t* react_box,
                                int32_t* out, int tc, int tc_defer, int current) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) {
    uint8_t f = p.flag[i];
    if (current) {
      int lag = 0;
      if (f & FLAG_PASSIVE) lag = tc;
      else if (!(f & (FLAG_INLIST | FLAG_FRESH | FLAG_HOME_SHELL))) lag = tc_defer + tc;
      else if (!(f & (FLAG_INLIST | FLAG_HOME_SHELL))) lag = tc;
      if (lag > 0) {
        uint32_t c = p.cell[i];
        T ox = p.ox[i], oy = p.oy[i], oz = p.oz[i], vx = p.vx[i], vy = p.vy[i], vz = p.vz[i];
        stream_one(kp, react_box, c, ox, oy, oz, vx, vy, vz, f, true, lag);
      }
    }
    out[lid ? lid[i] : i] = f & FLAG_SPECIES;
  }
}

template <typename T>
void Launch<T>::download_flag(const Dev<T>& d, const KParams<T>& kp, int32_t* out, int tc, int tc_defer,
                              int current, cudaStream_t st) {
  k_download_flag<T><<<1024, TPB, 0, st>>>(d.p, d.lid, kp, d.react_box, out, tc, tc_defer, current);
  LAUNCH_COUNT();
}

// ------------------------------------------------------------- spheres ----
template <typename T>
__global__ void k_srel(Dev<T> d, KParams<T> kp) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= kp.ns) return;
  SphereRel<T> r;
  double X = d.dpos[3 * s], Y = d.dpos[3 * s + 1], Z = d.dpos[3 * s + 2];
  double fx = floor(X), fy = floor(Y), fz = floor(Z);
  r.cx = (int)fx; r.cy = (int)fy; r.cz = (int)fz;
  r.ox = (T)(X - fx); r.oy = (T)(Y - fy); r.oz = (T)(Z - fz);
  d.srel[s] = r;
}

template <typename T>
void Launch<T>::update_srel(const Dev<T>& d, const KParams<T>& kp, cudaStream_t st) {
  if (kp.ns == 0) return;
  k_srel<T><<<(kp.ns + 127) / 128, 128, 0, st>>>(d, kp);
  LAUNCH_COUNT();
}

// Coarse bins of BIN_EDGE^3 cells listing the spheres whose (cutoff + skin)
// ball reaches into the bin; they replace the O(N * spheres) scan of
// neighbour_list_mod.f95:38-57 by an O(1) candidate lookup per particle.
// Cell range of a sphere's influence ball along one axis: [lo, hi] after
// clamping (walls) or, when the ball spans the whole periodic axis, the full
// axis without wrap.  Returns whether the range wraps.
__device__ __forceinline__ bool axis_range(double X, double R, int L, bool periodic, int& lo, int& hi) {
  lo = (int)floor(X - R);
  hi = (int)floor(X + R);
  if (!periodic) {
    lo = max(lo, 0);
    hi = min(hi, L - 1);
    return false;
  }
  if (hi - lo + 1 >= L) { lo = 0; hi = L - 1; return false; }
  return true;
}

__device__ __forceinline__ int wrap_mod(int c, int L) {
  c %= L;
  return c < 0 ? c + L : c;
}

// Cell c of the range [lo, hi] stands for its coarse bin when it is the first
// cell of the range inside that bin; the only bin a wrapped range can enter
// twice is the bin of lo.
__device__ __forceinline__ bool bin_first(int c, int lo, int L, bool wraps, int& bin) {
  int cc = wraps ? wrap_mod(c, L) : c;
  bin = cc / BIN_EDGE;
  if (c == lo) return true;
  int pc = wraps ? wrap_mod(c - 1, L) : c - 1;
  if (pc / BIN_EDGE == bin) return false;
  if (wraps && wrap_mod(lo, L) / BIN_EDGE == bin) return false;
  return true;
}

// Bins along one axis: box edges are at most 1024 cells, bins BIN_EDGE wide.
constexpr int MAX_BINS_PER_AXIS = 1024 / BIN_EDGE;

template <typename T>
__global__ void k_bins_fill(Dev<T> d, KParams<T> kp, double Rc, double Rn, int tc_defer) {
  const int s = blockIdx.x;
  if (s >= kp.ns) return;
  double R = (s & 1) ? Rn : Rc;
  if (tc_defer > 0) {
    // the farthest a deferred particle can be from its stored position: its
    // speed is bounded by the last rebuild's maximum or, after a collision,
    // by the maximum over the rotated outside particles; plus one cell for
    // the in-cell offset
    const double v2 = fmax(__longlong_as_double((long long)d.ctr->vlast),
                           __longlong_as_double((long long)d.ctr->vpost));
    R += sqrt(v2) * kp.dtd * (double)tc_defer + 1.0;
  }
  if (threadIdx.x == 0) {
    const double* V = d.dvel + 3 * s;
    atomicMax(&d.ctr->vsph, ord_bits(sqrt(V[0] * V[0] + V[1] * V[1] + V[2] * V[2])));
  }
  // per axis, the bins the cell range [lo, hi] enters (each once), listed by
  // one thread each; then one thread per bin of the product
  __shared__ int16_t blist[3][MAX_BINS_PER_AXIS];
  __shared__ int nbl[3];
  if (threadIdx.x < 3) {
    const int q = threadIdx.x;
    const int L = q == 0 ? kp.lx : (q == 1 ? kp.ly : kp.lz);
    const bool per = q < 2 || kp.geometry == 1;
    int lo, hi;
    const bool wr = axis_range(d.dpos[3 * s + q], R, L, per, lo, hi);
    int m = 0;
    for (int c = lo; c <= hi; ++c) {
      int b;
      if (bin_first(c, lo, L, wr, b) && m < MAX_BINS_PER_AXIS) blist[q][m++] = (int16_t)b;
    }
    nbl[q] = m;
  }
  __syncthreads();
  const int nx = nbl[0], ny = nbl[1], nz = nbl[2];
  const int tot = nx * ny * nz;
  const int nbins = kp.nbx * kp.nby * kp.nbz;
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    const int bx = blist[0][t % nx], by = blist[1][(t / nx) % ny], bz = blist[2][t / (nx * ny)];
    int bin = bx + kp.nbx * (by + kp.nby * bz);
    if (!chk(bin >= 0 && bin < nbins, d.ctr, 108, bin)) continue;
    unsigned int slot = atomicAdd(&d.bin_cnt[bin], 1u);
    if (slot < (unsigned)BIN_SLOTS) d.bin_list[(size_t)bin * BIN_SLOTS + slot] = (uint16_t)s;
    else atomicOr(&d.ctr->status, DEV_ERR_BIN_OVERFLOW);
  }
}

// Sorts each bin's list and writes the bitmask of the bins that list a sphere
// (one word per 32 consecutive bins, from the warp's ballot).
template <typename T>
__global__ void k_bins_sort(Dev<T> d, int nbins) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned int n = 0u;
  if (b < nbins) {
    n = min(d.bin_cnt[b], (unsigned)BIN_SLOTS);
    uint16_t* l = d.bin_list + (size_t)b * BIN_SLOTS;
    for (unsigned int i = 1; i < n; ++i) {
      uint16_t v = l[i];
      int j = (int)i - 1;
      while (j >= 0 && l[j] > v) { l[j + 1] = l[j]; --j; }
      l[j + 1] = v;
    }
    if (n < d.bin_cnt[b]) d.bin_cnt[b] = n;
  }
  const unsigned m = __ballot_sync(0xffffffffu, n > 0u);
  if ((threadIdx.x & 31) == 0 && b < nbins) d.bin_mask[b >> 5] = m;
}

template <typename T>
void Launch<T>::build_bins(const Dev<T>& d, const KParams<T>& kp, int tc_defer, cudaStream_t st) {
  int nbins = kp.nbx * kp.nby * kp.nbz;
  cudaMemsetAsync(d.bin_cnt, 0, sizeof(uint32_t) * nbins, st);
  if (kp.ns == 0) {
    cudaMemsetAsync(d.bin_mask, 0, sizeof(uint32_t) * ((nbins + 31) / 32), st);
    return;
  }
  double Rc = sqrt((double)kp.full2[0]) + 1e-6, Rn = sqrt((double)kp.full2[1]) + 1e-6;
  k_bins_fill<T><<<kp.ns, 128, 0, st>>>(d, kp, Rc, Rn, tc_defer);
  k_bins_sort<T><<<(nbins + 255) / 256, 256, 0, st>>>(d, nbins);
  LAUNCH_COUNT(); LAUNCH_COUNT();
}

__device__ __forceinline__ int bin_of(int lx, int ly, int nbx, int nby, uint32_t cell) {
  return cell_x(cell) / BIN_EDGE + nbx * (cell_y(cell) / BIN_EDGE + nby * (cell_z(cell) / BIN_EDGE));
}

// Gap-field bin of a cell (GAP_EDGE cells per bin edge).
__device__ __forceinline__ int gap_bin_of(int ngx, int ngy, uint32_t cell) {
  return cell_x(cell) / GAP_EDGE + ngx * (cell_y(cell) / GAP_EDGE + ngy * (cell_z(cell) / GAP_EDGE));
}

// Bins whose bitmask fits in shared memory (32 KB: a 256^3-cell box).
constexpr int BIN_MASK_SMEM_WORDS = 8192;

// Free-flight test of a shell member.  The reference integrates every member
// of its inside list each MD step (evolve_mod.f95:225-316).  A member that,
// at its constant velocity, cannot come within an LJ cutoff of a listed sphere
// (the spheres moving at most vs) before the next collision rebuild, cannot
// hit a wall and cannot reach the displacement criterion gets no force and no
// kick until then, so the engine streams it lazily instead (same positions up
// to rounding).  min_gap is the smallest distance beyond the cutoff over its
// listed spheres.
template <typename T>
__device__ __forceinline__ bool free_flight_ok(const KParams<T>& kp, uint32_t cell, T oz, T vx, T vy, T vz, T msd,
                                               T min_gap, int horizon, T vs) {
  const T v2 = vx * vx + vy * vy + vz * vz;
  const T t = kp.dt * (T)horizon;
  const T reach = (sqrt(v2) + vs) * t + (T)0.1;
  if (!(min_gap > reach)) return false;
  if (!(msd + (T)horizon * v2 * (kp.dt * kp.dt) < kp.msd_thr)) return false;
  if (kp.geometry == 0) {
    const T z0 = (T)cell_z(cell) + oz, z1 = z0 + vz * t;
    const T lo = (T)0.05, hi = (T)kp.lz - (T)0.05;
    if (!(z0 > lo && z0 < hi && z1 > lo && z1 < hi)) return false;
  }
  return true;
}

// Bound on the sphere speeds over the next collision period: twice the
// largest speed seen so far plus a margin.
template <typename T>
__device__ __forceinline__ T sphere_speed_bound(const Counters* c) {
  return (T)(2.0 * __longlong_as_double((long long)c->vsph) + 0.05);
}

// ------------------------------------------------------------- rebuild ----
// One pass over all particles at a neighbour-list rebuild
// (evolve_mod.f95:465-564): lazy streaming of the outside particles by
// time_count steps, merge of the shell buffer, shell membership and sphere
// pairs for every particle (neighbour_list + inout_particle_list), max v^2 for
// time_penetrate, and on collision steps the collision and distribute
// accumulation of the particles that stay outside.
template <typename T>
__global__ void __launch_bounds__(TPB, 4) k_rebuild(Dev<T> d, KParams<T> kp, StepArgs a) {
  if (d.ctr->abort_step) return;
  const T sx = step_shift<T>(a, 0), sy = step_shift<T>(a, 1), sz = step_shift<T>(a, 2);
  T vmax2 = (T)0;
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // warp-aligned grid-stride loop: the distribute counts are aggregated over
  // the lanes of a warp that fall in the same cell
  unsigned int pend_old = 0, pend_shift = 0, pend_cnt = 0;
  // The main-array state of the next iteration is loaded before the current
  // one is processed, so that two iterations' loads are in flight.
  // A rebuild between full passes with a valid watch list visits only the
  // particles on it: no other particle can enter a list or hit a wall before
  // the next collision, and their largest speed is kept in vfar.
  // The second half of a split collision pass (a.near) visits the particles
  // the far pass deferred, listed in the same buffer.
  const bool listed = a.use_watch || a.near;
  const int64_t nloop = a.near ? (int64_t)d.ctr->n_near : (a.use_watch ? (int64_t)d.ctr->n_watch : kp.n);
  // sphere speed bound of the free-flight test, read once (FP64 arithmetic
  // is slow on this part)
  const T vs_bound = (a.horizon > 0 && !a.mpc) ? sphere_speed_bound<T>(d.ctr) : (T)0;
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&d.ctr->acc_rebuild, (unsigned long long)nloop);
  auto pidx = [&](int64_t k) -> int64_t { return listed ? (int64_t)d.watch[k] : k; };
  const int64_t first = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31) + lane;
  uint8_t pf_f = 0;
  uint32_t pf_cell = 0, pf_lid = 0;   // (the main index only after a re-sort)
  T pf_ox = 0, pf_oy = 0, pf_oz = 0, pf_vx = 0, pf_vy = 0, pf_vz = 0;
  // (the species lists of a collision step need it for every particle; a
  // placed shell member of another rebuild loads its own)
  const bool want_lid = d.lid && a.mpc && kp.kinetics != 0 && !a.merge_only;
  if (first < nloop) {
    const int64_t q = pidx(first);
    pf_f = d.p.flag[q]; pf_cell = d.p.cell[q];
    pf_ox = d.p.ox[q]; pf_oy = d.p.oy[q]; pf_oz = d.p.oz[q];
    pf_vx = d.p.vx[q]; pf_vy = d.p.vy[q]; pf_vz = d.p.vz[q];
    if (want_lid) pf_lid = d.lid[q];
  }
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < nloop; base += stride) {
    const int64_t k = base + lane;
    const int64_t i = k < nloop ? pidx(k) : kp.n;
    bool dist = false;
    uint32_t cid = 0;
    uint8_t sp = 0;
    uint8_t f = pf_f;
    uint32_t cell = pf_cell;
    const uint32_t my_lid = want_lid ? pf_lid : (uint32_t)i;
    T ox = pf_ox, oy = pf_oy, oz = pf_oz;
    T vx = pf_vx, vy = pf_vy, vz = pf_vz;
    const int64_t knext = k + stride;
    if (knext < nloop) {
      const int64_t q = pidx(knext);
      pf_f = d.p.flag[q]; pf_cell = d.p.cell[q];
      pf_ox = d.p.ox[q]; pf_oy = d.p.oy[q]; pf_oz = d.p.oz[q];
      pf_vx = d.p.vx[q]; pf_vy = d.p.vy[q]; pf_vz = d.p.vz[q];
      if (want_lid) pf_lid = d.lid[q];
    }
    if (k < nloop) {
      const uint32_t cell0 = cell;
      const T vx0 = vx, vy0 = vy, vz0 = vz;
      const bool from_shell = (f & FLAG_HOME_SHELL) != 0;
      // lag of a main-home state: written at the last rebuild (fresh or free
      // flight) or at the last full pass (deferred); a flushed shell state is current
      int lag = 0;
      if (!from_shell && !(f & FLAG_INLIST)) lag = (f & (FLAG_FRESH | FLAG_PASSIVE)) ? a.tc : a.tc_full;
      const bool deferred = !from_shell && !(f & (FLAG_INLIST | FLAG_FRESH | FLAG_PASSIVE));
      const bool streamed = lag > 0;
      bool skip = false;
      // Fast path of a rebuild between full passes: a deferred particle whose
      // stored bin reaches no sphere (the bins are widened by the largest
      // flight since the full pass) and whose flight hits no wall can be
      // neither in a list nor written; only its speed counts.
      if (!a.full && deferred) {
        const bool nosph = kp.ns == 0 || d.bin_cnt[bin_of(kp.lx, kp.ly, kp.nbx, kp.nby, cell)] == 0u;
        bool nowall = true;
        if (kp.geometry == 0) {
          const T z = (T)cell_z(cell) + oz + vz * (kp.dt * (T)a.tc_full);
          nowall = z > (T)1e-3 && z < (T)kp.lz - (T)1e-3;
        }
        skip = nosph && nowall;
      }
      if (f & FLAG_HOME_SHELL) {
        uint32_t j = cell;
        if (!chk((int64_t)j < d.sh.cap, d.ctr, 109, j)) { skip = true; j = 0; }
        cell = d.sh.cell[j];
        ox = d.sh.ox[j]; oy = d.sh.oy[j]; oz = d.sh.oz[j];
        vx = d.sh.vx[j]; vy = d.sh.vy[j]; vz = d.sh.vz[j];
        sp = d.sh.flag[j] & FLAG_SPECIES;
      } else {
        sp = f & FLAG_SPECIES;
        if (streamed && !skip) {
          uint8_t ff = sp;
          stream_one(kp, d.react_box, cell, ox, oy, oz, vx, vy, vz, ff, true, lag);
          sp = ff & FLAG_SPECIES;
        }
      }
      T v2 = vx * vx + vy * vy + vz * vz;
      vmax2 = v2 > vmax2 ? v2 : vmax2;
      // write back only what changed: a state merged from the shell in full;
      // a lazily streamed particle its offsets, and its cell, velocity (wall
      // bounce) and flag when they changed
      const bool wr_all = from_shell;
      const bool wr_cell = wr_all || cell != cell0;
      const bool wr_pos = wr_all || streamed;
      const bool wr_vel = wr_all || vx != vx0 || vy != vy0 || vz != vz0;
      const bool wr_flag = wr_all || sp != f;
      if (skip) {
      } else if (a.merge_only) {
        if (wr_cell) d.p.cell[i] = cell;
        if (wr_pos) { d.p.ox[i] = ox; d.p.oy[i] = oy; d.p.oz[i] = oz; }
        if (wr_vel) { d.p.vx[i] = vx; d.p.vy[i] = vy; d.p.vz[i] = vz; }
        if (wr_flag) d.p.flag[i] = sp;
      } else {
        // candidate spheres of this particle's coarse bin
        int np = 0;
        bool nonbulk = false;
        T min_gap = (T)1e30;
        // sphere ids of the pairs, 16 bits per slot packed in two registers
        // (slots 0-3 and 4-7; 0xFFFF = empty), no indexed local array
        unsigned long long slo = ~0ull, shi = ~0ull;
        if (kp.ns > 0) {
          int bin = bin_of(kp.lx, kp.ly, kp.nbx, kp.nby, cell);
          bool okb = chk(bin >= 0 && bin < kp.nbx * kp.nby * kp.nbz, d.ctr, 110, (long long)cell);
          unsigned int nc = okb ? d.bin_cnt[bin] : 0u;
          if (!chk(nc <= (unsigned)BIN_SLOTS, d.ctr, 111, nc)) nc = 0;
          const uint16_t* bl = d.bin_list + (size_t)(okb ? bin : 0) * BIN_SLOTS;
          for (unsigned int q = 0; q < nc; ++q) {
            int s = bl[q];
            if (!chk(s < kp.ns, d.ctr, 112, s)) continue;
            SphereRel<T> sr = d.srel[s];
            T dx, dy, dz;
            T d2 = sep2(kp, cell, ox, oy, oz, sr, dx, dy, dz);
            if (d2 <= kp.full2[s & 1]) {
              if (np < PAIRMAX) {
                const int sh = 16 * (np & 3);
                const unsigned long long m = ~(0xFFFFull << sh), v = (unsigned long long)(uint16_t)s << sh;
                if (np < 4) slo = (slo & m) | v;
                else shi = (shi & m) | v;
              }
              np++;
              if (d2 <= kp.cut2[s & 1]) nonbulk = true;
              if (a.horizon > 0) {
                const T gap = sqrt(d2) - sqrt(kp.cut2[s & 1]);
                min_gap = gap < min_gap ? gap : min_gap;
              }
            }
          }
        }
        if (np > PAIRMAX) { atomicOr(&d.ctr->status, DEV_ERR_PAIR_OVERFLOW); np = PAIRMAX; }
        // a free-flight member must not have entered a cutoff since it was classified
        if ((f & FLAG_PASSIVE) && nonbulk) atomicOr(&d.ctr->status, DEV_ERR_PASSIVE);
        // (catalysis on exit: a particle inside a C cutoff at the last
        // force evaluation stays in the shell until one finds it outside)
        const bool passive = np > 0 && a.horizon > 0 && !a.mpc && !(d.inc && d.inc[i]) &&
                             free_flight_ok(kp, cell, oz, vx, vy, vz, (T)0, min_gap, a.horizon, vs_bound);
        const uint8_t nf = passive ? (uint8_t)(sp | FLAG_PASSIVE) : sp;
        bool placed = false;
        if (np > 0 && !passive) {
          cg::coalesced_group g = cg::coalesced_threads();
          unsigned int bslot = 0;
          if (g.thread_rank() == 0) bslot = atomicAdd(&d.ctr->n_inside_new, g.size());
          bslot = g.shfl(bslot, 0);
          unsigned int j = bslot + g.thread_rank();
          if ((int64_t)j >= d.sh2.cap) {
            atomicOr(&d.ctr->status, DEV_ERR_SHELL_OVERFLOW);
          } else {
            d.sh2.idx[j] = (uint32_t)i;
            d.sh2.mid[j] = want_lid ? my_lid : lid_of(d, (uint32_t)i);
            d.sh2.cell[j] = cell;
            d.sh2.ox[j] = ox; d.sh2.oy[j] = oy; d.sh2.oz[j] = oz;
            d.sh2.vx[j] = vx; d.sh2.vy[j] = vy; d.sh2.vz[j] = vz;
            d.sh2.msd[j] = (T)0;
            d.sh2.flag[j] = sp | FLAG_INLIST;
            d.sh2.nonbulk[j] = nonbulk ? 1 : 0;
            d.sh2.np[j] = (uint8_t)np;
            uint4 packed;
            packed.x = (uint32_t)slo; packed.y = (uint32_t)(slo >> 32);
            packed.z = (uint32_t)shi; packed.w = (uint32_t)(shi >> 32);
            *reinterpret_cast<uint4*>(d.sh2.sph + (size_t)j * PAIRMAX) = packed;
            d.p.cell[i] = j;
            d.p.flag[i] = sp | FLAG_INLIST | FLAG_HOME_SHELL;
            placed = true;
          }
        }
        // A rebuild between full passes leaves a deferred outside particle
        // unwritten (its lazy stream waits for the next full pass) unless its
        // flight hit a wall; everything else it writes is marked fresh.
        const bool keep = !placed && !a.full && deferred && !passive && !wr_vel && sp == (f & FLAG_SPECIES);
        if (!placed && !keep) {
          const uint8_t nf2 = (a.full || passive) ? nf : (uint8_t)(nf | FLAG_FRESH);
          if (wr_cell) d.p.cell[i] = cell;
          if (wr_pos) { d.p.ox[i] = ox; d.p.oy[i] = oy; d.p.oz[i] = oz; }
          if (wr_vel) { d.p.vx[i] = vx; d.p.vy[i] = vy; d.p.vz[i] = vz; }
          if (wr_all || nf2 != f) d.p.flag[i] = nf2;
        }
        if (!placed) {
          if (a.mpc) {
            uint32_t key = shifted_key(kp, cell, ox, oy, oz, sx, sy, sz);
            d.skey[i] = key;
            accum_coll<T>(d.acc, key, vx, vy, vz);
            dist = kp.kinetics != 0;
            cid = unshifted_id(kp.lx, kp.ly, cell);
          }
        }
      }
    }
    // distribute_mod.f95:95-182 counts and first members, one atomic per
    // (cell, species) group of the warp; the group's lowest lane holds its
    // smallest particle index
    if (a.mpc && kp.kinetics != 0 && !a.merge_only) {
      // 32-bit key (cid < 2^30 since every box edge is at most 1024 cells);
      // a 64-bit match costs twice the SM cycles of a 32-bit one
      const unsigned dmask = __ballot_sync(0xffffffffu, dist);
      unsigned peers = 0u;
      if (dist) peers = __match_any_sync(dmask, (cid << 2) | (uint32_t)sp);
      // a listed pass holds its particles in list order, and re-sorted slots
      // are not in index order: the group's smallest index is reduced over
      // its lanes
      uint32_t first_i = dist ? my_lid : 0u;
      if (dist && (listed || d.lid)) first_i = __reduce_min_sync(peers, first_i);
      if (dist && lane == __ffs(peers) - 1) {
        // the count returned by this atomic is checked one iteration later,
        // so that the warp does not wait for it
        if (pend_cnt && ((pend_old >> pend_shift) & 255u) + pend_cnt > (unsigned)kp.cell_capacity)
          atomicOr(&d.ctr->status, DEV_ERR_CELL_OVERFLOW);
        pend_cnt = __popc(peers);
        pend_shift = 8 * sp;
        pend_old = atomicAdd(&d.dcnt[cid], pend_cnt << pend_shift);
        atomicMin(&d.dfirst[4 * (size_t)cid + sp], dist_key(0, first_i));
      }
    }
  }
  if (pend_cnt && ((pend_old >> pend_shift) & 255u) + pend_cnt > (unsigned)kp.cell_capacity)
    atomicOr(&d.ctr->status, DEV_ERR_CELL_OVERFLOW);
  if (a.use_watch && blockIdx.x == 0 && threadIdx.x == 0) atomicMax(&d.ctr->maxv2, d.ctr->vfar);
  block_max_to<T>(&d.ctr->maxv2, vmax2);
}

// First half of a split collision-step full pass (evolve_mod.f95:465-564 with
// the collision and distribute accumulation, as k_rebuild with a.full and
// a.mpc).  It handles the particles that need no list work: an outside state
// whose lazily streamed position is beyond the list radius of every sphere of
// its coarse bin enters no shell list, so it is streamed, written, and
// accumulated here with no shell placement or shell-buffer state in the
// kernel.  Every other particle (a state in the shell buffer, or within a
// list radius) is left untouched and appended to the near list (d.watch,
// n_near, staged per warp in shared memory), which k_rebuild then processes
// in full.
template <typename T>
__global__ void __launch_bounds__(TPB, 4) k_rebuild_far(Dev<T> d, KParams<T> kp, StepArgs a) {
  if (d.ctr->abort_step) return;
  const T sx = step_shift<T>(a, 0), sy = step_shift<T>(a, 1), sz = step_shift<T>(a, 2);
  T vmax2 = (T)0;
  const int lane = threadIdx.x & 31;
  unsigned int pend_old = 0, pend_shift = 0, pend_cnt = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&d.ctr->acc_rebuild, (unsigned long long)kp.n);
  const bool distrib = kp.kinetics != 0;
  // the bitmask of the bins that list a sphere, in shared memory when it fits:
  // most particles are far from every sphere and skip the bin-count load
  __shared__ uint32_t smask[BIN_MASK_SMEM_WORDS];
  const int nmask = (kp.nbx * kp.nby * kp.nbz + 31) / 32;
  const bool use_smask = kp.ns > 0 && nmask <= BIN_MASK_SMEM_WORDS;
  if (use_smask) {
    for (int w = threadIdx.x; w < nmask; w += blockDim.x) smask[w] = d.bin_mask[w];
    __syncthreads();
  }
  __shared__ uint32_t s_gmin[TPB];   // per-warp group minima of the main index (after a re-sort)
  __shared__ uint32_t wl_buf[(TPB / 32) * WL_CAP];
  uint32_t* wbuf = wl_buf + (threadIdx.x >> 5) * WL_CAP;
  unsigned wn = 0;
  // Blocks take tiles of FAR_TILE consecutive particles in a grid stride,
  // the warps of a block interleaved in 32-particle steps inside a tile: the
  // GPU still sweeps the arrays front to back, and the near list a warp
  // stages holds particles of one tile at a time, so the shell built from it
  // keeps their spatial (cell) order.
  // (32-bit indices: particle counts are below 2^31, and an index plus one
  // tile stride stays below 2^32)
  constexpr int FAR_STEPS = 8;    // 2048-particle tiles (4096 and 1024 measured slower at 256^3)
  constexpr uint32_t FAR_TILE = (uint32_t)FAR_STEPS * TPB;
  const uint32_t n32 = (uint32_t)kp.n;
  const uint32_t tile_stride = gridDim.x * FAR_TILE;
  uint32_t i = blockIdx.x * FAR_TILE + threadIdx.x;
  int step = 0;
  auto advance = [&](uint32_t j, int st) -> uint32_t {   // the index after j (at step st of its tile)
    return st + 1 < FAR_STEPS ? j + TPB : j - (uint32_t)(FAR_STEPS - 1) * TPB + tile_stride;
  };
  uint8_t pf_f = FLAG_HOME_SHELL;
  uint32_t pf_cell = 0, pf_lid = 0;   // (the main index only after a re-sort)
  T pf_ox = 0, pf_oy = 0, pf_oz = 0, pf_vx = 0, pf_vy = 0, pf_vz = 0;
  if (i < n32) {
    pf_f = d.p.flag[i]; pf_cell = d.p.cell[i];
    pf_ox = d.p.ox[i]; pf_oy = d.p.oy[i]; pf_oz = d.p.oz[i];
    pf_vx = d.p.vx[i]; pf_vy = d.p.vy[i]; pf_vz = d.p.vz[i];
    if (distrib && d.lid) pf_lid = d.lid[i];
  }
  // the loop runs while the warp's step base is inside the array (warp-uniform)
  for (; i - lane < n32; i = advance(i, step), step = step + 1 < FAR_STEPS ? step + 1 : 0) {
    const bool in = i < n32;
    const uint8_t f = pf_f;
    uint32_t cell = pf_cell;
    const uint32_t my_lid = pf_lid;
    T ox = pf_ox, oy = pf_oy, oz = pf_oz;
    T vx = pf_vx, vy = pf_vy, vz = pf_vz;
    const uint32_t inext = advance(i, step);
    if (inext < n32) {
      pf_f = d.p.flag[inext]; pf_cell = d.p.cell[inext];
      pf_ox = d.p.ox[inext]; pf_oy = d.p.oy[inext]; pf_oz = d.p.oz[inext];
      pf_vx = d.p.vx[inext]; pf_vy = d.p.vy[inext]; pf_vz = d.p.vz[inext];
      if (distrib && d.lid) pf_lid = d.lid[inext];
    }
    bool far = in && !(f & FLAG_HOME_SHELL);
    bool near = in && !far;
    uint8_t sp = f & FLAG_SPECIES;
    uint32_t cid = 0;
    if (far) {
      const uint32_t cell0 = cell;
      const T vx0 = vx, vy0 = vy, vz0 = vz;
      int lag = 0;
      if (!(f & FLAG_INLIST)) lag = (f & (FLAG_FRESH | FLAG_PASSIVE)) ? a.tc : a.tc_full;
      if (lag > 0) {
        uint8_t ff = sp;
        stream_one(kp, d.react_box, cell, ox, oy, oz, vx, vy, vz, ff, true, lag);
        sp = ff & FLAG_SPECIES;
      }
      // within the list radius of a sphere of its bin: the whole particle
      // goes to k_rebuild (lists, shell placement)
      const int bin = bin_of(kp.lx, kp.ly, kp.nbx, kp.nby, cell);
      if (kp.ns > 0 && (!use_smask || ((smask[bin >> 5] >> (bin & 31)) & 1u))) {
        unsigned int nc = d.bin_cnt[bin];
        nc = nc < (unsigned)BIN_SLOTS ? nc : (unsigned)BIN_SLOTS;
        const uint16_t* bl = d.bin_list + (size_t)bin * BIN_SLOTS;
        for (unsigned int q = 0; q < nc && !near; ++q) {
          const int sph = bl[q];
          T dx, dy, dz;
          if (sep2(kp, cell, ox, oy, oz, d.srel[sph], dx, dy, dz) <= kp.full2[sph & 1]) near = true;
        }
        far = !near;
      }
      if (far) {
        const T v2 = vx * vx + vy * vy + vz * vz;
        vmax2 = v2 > vmax2 ? v2 : vmax2;
        if (cell != cell0) d.p.cell[i] = cell;
        if (lag > 0) { d.p.ox[i] = ox; d.p.oy[i] = oy; d.p.oz[i] = oz; }
        if (vx != vx0 || vy != vy0 || vz != vz0) { d.p.vx[i] = vx; d.p.vy[i] = vy; d.p.vz[i] = vz; }
        if (sp != f) d.p.flag[i] = sp;
        const uint32_t key = shifted_key(kp, cell, ox, oy, oz, sx, sy, sz);
        d.skey[i] = key;
        accum_coll<T>(d.acc, key, vx, vy, vz);
        cid = unshifted_id(kp.lx, kp.ly, cell);
      }
    }
    wl_add(wbuf, wn, near, (uint32_t)i, &d.ctr->n_near, d.watch);
    // distribute_mod.f95:95-182 counts and first members as in k_rebuild
    if (distrib) {
      const bool dist = far;
      const unsigned dmask = __ballot_sync(0xffffffffu, dist);
      unsigned peers = 0u;
      if (dist) peers = __match_any_sync(dmask, (cid << 2) | (uint32_t)sp);
      // the group's lowest lane holds its smallest index unless re-sorted
      // slots put the indices out of order; then the group's lanes take the
      // minimum at their leader's slot of a per-warp table in shared memory
      // (convergent; a reduction over each group's own mask serialises the
      // groups and cost a sixth of the pass)
      uint32_t first_i = (uint32_t)i;
      if (d.lid) {
        uint32_t* gmin = s_gmin + (threadIdx.x & ~31);
        gmin[lane] = 0xFFFFFFFFu;
        __syncwarp();
        if (dist) atomicMin(&gmin[__ffs(peers) - 1], my_lid);
        __syncwarp();
        first_i = gmin[lane];
        __syncwarp();
      }
      if (dist && lane == __ffs(peers) - 1) {
        if (pend_cnt && ((pend_old >> pend_shift) & 255u) + pend_cnt > (unsigned)kp.cell_capacity)
          atomicOr(&d.ctr->status, DEV_ERR_CELL_OVERFLOW);
        pend_cnt = __popc(peers);
        pend_shift = 8 * sp;
        pend_old = atomicAdd(&d.dcnt[cid], pend_cnt << pend_shift);
        atomicMin(&d.dfirst[4 * (size_t)cid + sp], dist_key(0, first_i));
      }
    }
  }
  wl_flush(wbuf, wn, &d.ctr->n_near, d.watch);
  if (pend_cnt && ((pend_old >> pend_shift) & 255u) + pend_cnt > (unsigned)kp.cell_capacity)
    atomicOr(&d.ctr->status, DEV_ERR_CELL_OVERFLOW);
  block_max_to<T>(&d.ctr->maxv2, vmax2);
}

template <typename T>
void Launch<T>::rebuild_split(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st) {
  cudaMemsetAsync(&d.ctr->n_near, 0, sizeof(unsigned int), st);
  k_rebuild_far<T><<<a.g_far, TPB, 0, st>>>(d, kp, a);
  StepArgs b = a;
  b.near = 1;
  b.use_watch = 0;
  k_rebuild<T><<<a.g_rebuild, TPB, 0, st>>>(d, kp, b);
  LAUNCH_COUNT(); LAUNCH_COUNT();
}

template <typename T>
void Launch<T>::rebuild(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st) {
  k_rebuild<T><<<a.g_rebuild, TPB, 0, st>>>(d, kp, a);
  LAUNCH_COUNT();
}

template <typename T>
__global__ void k_finalize(Dev<T> d, KParams<T> kp, StepArgs a, double skin) {
  if (d.ctr->abort_step) return;
  double maxt = __longlong_as_double((long long)d.ctr->maxv2);
  d.ctr->time_penetrate = (int)floor((0.5 * skin / sqrt(maxt)) / kp.dtd);
  d.ctr->vlast = d.ctr->maxv2;
  if (a.mpc) d.ctr->vpost = 0ull;
  d.ctr->maxv2 = 0ull;
  d.ctr->maxmsd[0] = 0ull;
  d.ctr->maxmsd[1] = 0ull;
  if (!a.merge_only) {
    unsigned int m = d.ctr->n_inside_new;
    if ((int64_t)m > d.sh2.cap) m = (unsigned int)d.sh2.cap;   // overflow is reported via status
    d.ctr->acc_placed += m;
    d.ctr->n_inside = m;
    d.ctr->n_inside_new = 0u;
  }
}

template <typename T>
void Launch<T>::finalize_rebuild(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, double skin,
                                 cudaStream_t st) {
  k_finalize<T><<<1, 1, 0, st>>>(d, kp, a, skin);
  LAUNCH_COUNT();
}

// k_force's sphere-sphere blocks: warps per sphere, spheres per block
constexpr int SPH_WARPS = 4;
constexpr int SPH_PER_BLOCK = (TPB / 32) / SPH_WARPS;

// --------------------------------------------------------------- forces ----
// Per shell particle and MD step (evolve_mod.f95:567-670 with
// forces_mod.f95:6-140): LJ force against each sphere of its pair list in
// sphere order with the catalytic conversion, the second half kick, and unless
// the step ends in a collision or a call boundary the first half kick and free
// flight of the next step (evolve_mod.f95:225-316) with its max_solvent_dist.
// Extra blocks after the shell grid compute the sphere-sphere LJ forces
// (forces_mod.f95:144-210) of the current sphere positions.
// OWN: the owner-tag form (a template flag: the common form keeps no tag state)
template <typename T, bool OWN>
__global__ void __launch_bounds__(TPB, sizeof(T) == 4 ? 5 : 1) k_force(Dev<T> d, KParams<T> kp, StepArgs a) {
  if (d.ctr->abort_step) return;
  if (!a.rebuilt) {
    // max_solvent_dist > threshold, compared on the double bits (both >= 0)
    const unsigned long long thr = (unsigned long long)__double_as_longlong(to_f64(kp.msd_thr));
    if (d.ctr->maxmsd[a.step & 1] > thr) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicCAS(&d.ctr->abort_step, 0, (int)a.step);
      return;
    }
  }
  if ((int)blockIdx.x >= a.g_force) {
    // sphere-sphere forces: SPH_WARPS warps per sphere s, each over every
    // SPH_WARPS-th group of 32 spheres, their sums added in warp order.  These
    // blocks start only as the shell blocks retire, so their latency adds to
    // the launch; a sphere's scan split four ways shortens it about fourfold.
    __shared__ double s_part[TPB / 32][4];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int part = wib % SPH_WARPS;
    const int sg = ((int)blockIdx.x - a.g_force) * SPH_PER_BLOCK + wib / SPH_WARPS;
    const bool have = sg < kp.ns;   // (warp-uniform)
    const int s = have ? sg : 0, ks = s >> 1, is = s & 1;
    const SphereRel<T> rs = d.srel[s];
    double fx = 0., fy = 0., fz = 0., pot = 0.;
    // (rotors have no motor-motor LJ: rotational_code/2d_array/evolve_mod.f95:515-531)
    const int nt = (kp.rotor || !have) ? 0 : kp.ns;
    bool hit = false;   // a pair within its cutoff on this lane
    for (int t = 32 * part + lane; t < nt; t += 32 * SPH_WARPS) {
      int kt = t >> 1, it = t & 1;
      if (kt == ks) continue;
      const SphereRel<T> rt = d.srel[t];
      int type = is + it;  // 0 CC, 1 CN, 2 NN
      float dxf = (float)(rs.cx - rt.cx) + (float)(rs.ox - rt.ox);
      float dyf = (float)(rs.cy - rt.cy) + (float)(rs.oy - rt.oy);
      float dzf = (float)(rs.cz - rt.cz) + (float)(rs.oz - rt.oz);
      dxf = min_image(dxf, (float)kp.Ld[0]);
      dyf = min_image(dyf, (float)kp.Ld[1]);
      if (kp.geometry == 1) dzf = min_image(dzf, (float)kp.Ld[2]);
      if (dxf * dxf + dyf * dyf + dzf * dzf > kp.mot_cut2f[type] * 1.001f + 1e-3f) continue;
      double dx = d.dpos[3 * s] - d.dpos[3 * t], dy = d.dpos[3 * s + 1] - d.dpos[3 * t + 1];
      double dz = d.dpos[3 * s + 2] - d.dpos[3 * t + 2];
      dx = min_image(dx, kp.Ld[0]);
      dy = min_image(dy, kp.Ld[1]);
      if (kp.geometry == 1) dz = min_image(dz, kp.Ld[2]);
      double dRsq = dx * dx + dy * dy + dz * dz;
      if (dRsq <= kp.mot_cut2[type]) {
        hit = true;
        double IdRsq = 1.0 / dRsq;
        double IdR6 = IdRsq * IdRsq * IdRsq, IdR8 = IdR6 * IdRsq, IdR12 = IdR6 * IdR6, IdR14 = IdR12 * IdRsq;
        double Fb = 4.0 * (kp.mot_r12R12[type] * IdR14 - kp.mot_r6R6[type] * IdR8);
        double Ub = 4.0 * (kp.mot_R12[type] * IdR12 - kp.mot_R6[type] * IdR6) + 1.0;
        fx += kp.em * Fb * dx;
        fy += kp.em * Fb * dy;
        fz += kp.em * Fb * dz;
        if (kt < ks) pot += kp.em * Ub;
      }
    }
    // a warp none of whose pairs is within its cutoff (nearly every warp:
    // the dimers are far apart) holds +0 everywhere and skips the FP64
    // reduction, which at GB300's FP64 rate made the tail of every step
    if (__any_sync(0xffffffffu, hit)) {
      for (int o = 16; o > 0; o >>= 1) {
        fx += __shfl_xor_sync(0xffffffffu, fx, o);
        fy += __shfl_xor_sync(0xffffffffu, fy, o);
        fz += __shfl_xor_sync(0xffffffffu, fz, o);
        pot += __shfl_xor_sync(0xffffffffu, pot, o);
      }
    }
    if (lane == 0) { s_part[wib][0] = fx; s_part[wib][1] = fy; s_part[wib][2] = fz; s_part[wib][3] = pot; }
    __syncthreads();
    if (have && part == 0 && lane < 4) {
      double v = 0.;
      for (int q = 0; q < SPH_WARPS; ++q) v += s_part[wib + q][lane];
      d.fmot[4 * s + lane] = v;
    }
    return;
  }
  const unsigned int nin = d.ctr->n_inside;
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&d.ctr->acc_force, (unsigned long long)nin);
  const int64_t stride = (int64_t)a.g_force * blockDim.x;
  const T sx = step_shift<T>(a, 0), sy = step_shift<T>(a, 1), sz = step_shift<T>(a, 2);
  const int lane = threadIdx.x & 31;
  T msdmax = (T)0;
  // warp-aligned grid-stride loop: a warp stays converged for the per-sphere
  // warp reductions below
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < (int64_t)nin; base += stride) {
    const int64_t j = base + lane;
    const bool act = j < (int64_t)nin;
    uint32_t cell = 0, idx = 0;
    T ox = 0, oy = 0, oz = 0, vx = 0, vy = 0, vz = 0;
    T msd0 = (T)0;   // loaded with the rest: its use at the end would wait on it
    uint8_t fl = 0;
    int np = 0;
    uint16_t sphl[PAIRMAX];
    if (act) {
      if (a.advance && !a.mpc) msd0 = d.sh.msd[j];
      cell = d.sh.cell[j];
      ox = d.sh.ox[j]; oy = d.sh.oy[j]; oz = d.sh.oz[j];
      vx = d.sh.vx[j]; vy = d.sh.vy[j]; vz = d.sh.vz[j];
      fl = d.sh.flag[j];
      np = d.sh.np[j];
      // the main index keys the catalysis draws and orders the species lists;
      // without owner tags or the on-exit record nothing here needs the slot,
      // so after a re-sort the entry's main index replaces it
      idx = (d.lid && !OWN && !d.inc) ? d.sh.mid[j] : d.sh.idx[j];
      const uint4 packed = *reinterpret_cast<const uint4*>(d.sh.sph + (size_t)j * PAIRMAX);
      sphl[0] = (uint16_t)(packed.x & 0xFFFFu); sphl[1] = (uint16_t)(packed.x >> 16);
      sphl[2] = (uint16_t)(packed.y & 0xFFFFu); sphl[3] = (uint16_t)(packed.y >> 16);
      sphl[4] = (uint16_t)(packed.z & 0xFFFFu); sphl[5] = (uint16_t)(packed.z >> 16);
      sphl[6] = (uint16_t)(packed.w & 0xFFFFu); sphl[7] = (uint16_t)(packed.w >> 16);
    }
    // owner tag (type_B) of the particle, with owner_tags
    uint32_t own = 0, own0 = 0;
    if (OWN && act) own = own0 = d.owner[idx];
    // The FP32 build sums an entry's pair forces for its two half kicks (and
    // stores the per-pair forces kept across a step boundary inside the
    // loop), which frees the per-slot registers; the FP64 parity build kicks
    // pair by pair in the reference's order (evolve_mod.f95:225-250, :645-670).
    constexpr bool SUMK = sizeof(T) == 4;
    const bool keep_pf = !(a.advance && !a.mpc);
    T fpx[PAIRMAX], fpy[PAIRMAX], fpz[PAIRMAX];
    T Fx = (T)0, Fy = (T)0, Fz = (T)0;
    bool anyC = false, inC = false;   // a C sphere listed / within its cutoff (catalysis on exit)
#pragma unroll
    for (int q = 0; q < PAIRMAX; ++q) {
      if (!SUMK) fpx[q] = fpy[q] = fpz[q] = (T)0;
      if (!__any_sync(0xffffffffu, q < np)) break;
      int s = (q < np) ? (int)sphl[q] : -1;
      T fx = 0, fy = 0, fz = 0, u = 0;
      if (s >= 0 && (s & 1) == 0) anyC = true;
      if (s >= 0) {
        const int t = s & 1;
        const SphereRel<T> sr = d.srel[s];
        T dx, dy, dz;
        T d2 = sep2(kp, cell, ox, oy, oz, sr, dx, dy, dz);
        if (d2 <= kp.cut2[t]) {
          int spc = fl & FLAG_SPECIES;
          T E = (t == 0) ? kp.eps_c[spc] : kp.eps_n[spc];
          if (OWN) {
            // linear_periodic_no_ci/forces_mod.f95:79-121: the C sphere of
            // motor k makes the particle a B of motor k; a B of another motor
            // acts as an A (the slots run in ascending sphere order, the
            // reference's motor loop)
            const uint32_t motor = (uint32_t)(s >> 1) + 1u;
            if (t == 0) { fl = (fl & ~FLAG_SPECIES) | 1; own = motor; E = kp.eps_c[1]; }
            else if (spc == 1 && own != motor) E = kp.eps_n[0];
          } else if (t == 0) {
            inC = true;
            if (kp.catalysis == 0) {
              if (spc == 0) { fl = (fl & ~FLAG_SPECIES) | 1; E = kp.eps_c[1]; }
            } else if (kp.catalysis == 1 && (spc == 0 || spc == 1)) {
              uint64_t m0, m1;
              contract_bits(kp.seed, TAG_CAT, (OWN || d.inc) ? lid_of(d, idx) : idx, (uint32_t)s, a.step, m0, m1);
              if (spc == 0 && m0 < kp.thr_ab) fl = (fl & ~FLAG_SPECIES) | 1;
              if (spc == 1 && m0 < kp.thr_ba) fl = (fl & ~FLAG_SPECIES) | 0;
            }
          }
          lj(kp, t, E, d2, dx, dy, dz, fx, fy, fz, u);
        } else {
          s = -1;   // in the skin only: no contribution
        }
      }
      if (SUMK) {
        Fx += fx; Fy += fy; Fz += fz;
        if (keep_pf && q < np) {
          const size_t bq = ((size_t)j * PAIRMAX + q) * 3;
          d.sh.pf[bq] = fx; d.sh.pf[bq + 1] = fy; d.sh.pf[bq + 2] = fz;
        }
      } else {
        fpx[q] = fx; fpy[q] = fy; fpz[q] = fz;
      }
      warp_sphere_add(d.facc, s, -fx, -fy, -fz, u);
    }
    if (act && !OWN && kp.catalysis == 2 && anyC) {
      // catalysis on exit: an A that was inside a C cutoff at the last force
      // evaluation and is outside every C cutoff now becomes a B (the pair
      // forces above use the species before the conversion); a restart's
      // force evaluation records the state only
      const bool was = d.inc[idx] != 0;
      if (was && !inC && !a.forces_only && (fl & FLAG_SPECIES) == 0) fl = (uint8_t)((fl & ~FLAG_SPECIES) | 1);
      if (was != inC) d.inc[idx] = inC ? 1 : 0;
    }
    if (act) {
      const T h2 = kp.hIM[fl & FLAG_SPECIES];
      if (SUMK) {
        if (!a.forces_only) { vx = vx + h2 * Fx; vy = vy + h2 * Fy; vz = vz + h2 * Fz; }
      } else {
#pragma unroll
        for (int q = 0; q < PAIRMAX; ++q) {
          if (q >= np || a.forces_only) break;
          vx = vx + h2 * fpx[q]; vy = vy + h2 * fpy[q]; vz = vz + h2 * fpz[q];
        }
      }
      if (a.mpc) {
        uint32_t key = shifted_key(kp, cell, ox, oy, oz, sx, sy, sz);
        d.sh.skey[j] = key;
        accum_coll<T>(d.acc, key, vx, vy, vz);
        if (kp.kinetics != 0) {
          bool bulk = kp.exclusion == 1 || !d.sh.nonbulk[j];
          if (bulk)
            accum_dist(d, kp, unshifted_id(kp.lx, kp.ly, cell), fl & FLAG_SPECIES,
                       dist_key(kp.exclusion == 0 ? 1 : 0, (OWN || d.inc) ? lid_of(d, idx) : idx));
        }
      }
      if (a.advance && !a.mpc) {
        if (SUMK) {
          vx = vx + h2 * Fx; vy = vy + h2 * Fy; vz = vz + h2 * Fz;
        } else {
#pragma unroll
          for (int q = 0; q < PAIRMAX; ++q) {
            if (q >= np) break;
            vx = vx + h2 * fpx[q]; vy = vy + h2 * fpy[q]; vz = vz + h2 * fpz[q];
          }
        }
        stream_one(kp, d.react_box, cell, ox, oy, oz, vx, vy, vz, fl, false, 1);
        T msd = msd0 + (vx * vx + vy * vy + vz * vz) * (kp.dt * kp.dt);
        d.sh.msd[j] = msd;
        msdmax = msd > msdmax ? msd : msdmax;
        d.sh.cell[j] = cell;
        d.sh.ox[j] = ox; d.sh.oy[j] = oy; d.sh.oz[j] = oz;
      } else if (!SUMK) {
#pragma unroll
        for (int q = 0; q < PAIRMAX; ++q) {
          if (q >= np) break;
          size_t bq = ((size_t)j * PAIRMAX + q) * 3;
          d.sh.pf[bq] = fpx[q]; d.sh.pf[bq + 1] = fpy[q]; d.sh.pf[bq + 2] = fpz[q];
        }
      }
      d.sh.vx[j] = vx; d.sh.vy[j] = vy; d.sh.vz[j] = vz;
      d.sh.flag[j] = fl;
      if (OWN && own != own0) d.owner[idx] = (uint16_t)own;
    }
  }
  if (a.advance && !a.mpc) block_max_to<T>(&d.ctr->maxmsd[(a.step + 1) & 1], msdmax);
}

template <typename T>
void Launch<T>::force(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st) {
  const int extra = (kp.ns + SPH_PER_BLOCK - 1) / SPH_PER_BLOCK;
  if (kp.owner_tags) k_force<T, true><<<a.g_force + extra, TPB, 0, st>>>(d, kp, a);
  else k_force<T, false><<<a.g_force + extra, TPB, 0, st>>>(d, kp, a);
  LAUNCH_COUNT();
}

// First half kick with the stored pair forces and free flight of the shell
// particles (evolve_mod.f95:225-316), used after a collision step or at the
// start of a run call; with rotate set it first applies the collision.
// With a.advance and a.horizon > 0 (right after a rebuild) it also sorts the
// shell: members that pass free_flight_ok move to the main home with
// FLAG_PASSIVE and their state of this step (they are streamed lazily from
// here), the others are streamed and packed into d.sh2, which the caller makes
// the current shell.
template <typename T>
__global__ void __launch_bounds__(TPB) k_shell_advance(Dev<T> d, KParams<T> kp, StepArgs a, int rotate) {
  const bool sort_shell = a.advance && a.horizon > 0;
  // (no displacement abort can be pending where the shell is sorted, and the
  // sorted buffer must be produced whatever happens)
  if (d.ctr->abort_step && !sort_shell) return;
  const unsigned int nin = d.ctr->n_inside;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const T vs = sphere_speed_bound<T>(d.ctr);
  T msdmax = (T)0;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < (int64_t)nin; j += stride) {
    T vx = d.sh.vx[j], vy = d.sh.vy[j], vz = d.sh.vz[j];
    if (rotate) {
      T r[6];
      load_rot(d.rot, d.sh.skey[j], r);
      rotate_v(kp, r, vx, vy, vz);
    }
    if (a.advance) {
      uint32_t cell = d.sh.cell[j];
      T ox = d.sh.ox[j], oy = d.sh.oy[j], oz = d.sh.oz[j];
      uint8_t fl = d.sh.flag[j];
      const int np = d.sh.np[j];
      const T h2 = kp.hIM[fl & FLAG_SPECIES];
      for (int q = 0; q < np; ++q) {
        size_t b = ((size_t)j * PAIRMAX + q) * 3;
        vx = vx + h2 * d.sh.pf[b]; vy = vy + h2 * d.sh.pf[b + 1]; vz = vz + h2 * d.sh.pf[b + 2];
      }
      if (sort_shell) {
        const uint4 packed = *reinterpret_cast<const uint4*>(d.sh.sph + (size_t)j * PAIRMAX);
        const uint16_t ids[PAIRMAX] = {
            (uint16_t)(packed.x & 0xFFFFu), (uint16_t)(packed.x >> 16), (uint16_t)(packed.y & 0xFFFFu),
            (uint16_t)(packed.y >> 16), (uint16_t)(packed.z & 0xFFFFu), (uint16_t)(packed.z >> 16),
            (uint16_t)(packed.w & 0xFFFFu), (uint16_t)(packed.w >> 16)};
        T min_gap = (T)1e30;
#pragma unroll
        for (int q = 0; q < PAIRMAX; ++q) {
          if (q >= np) break;
          const int s = ids[q];
          if (!chk(s < kp.ns, d.ctr, 121, s)) { min_gap = (T)-1; break; }
          T dx, dy, dz;
          const T d2 = sep2(kp, cell, ox, oy, oz, d.srel[s], dx, dy, dz);
          const T gap = sqrt(d2) - sqrt(kp.cut2[s & 1]);
          min_gap = gap < min_gap ? gap : min_gap;
        }
        const uint32_t idx = d.sh.idx[j];
        if (a.watch_build) watch_append(&d.ctr->n_watch, d.watch, idx);
        const T msd_now = d.sh.msd[j];
        if (!(d.inc && d.inc[idx]) && free_flight_ok(kp, cell, oz, vx, vy, vz, msd_now, min_gap, a.horizon, vs)) {
          // state of this step into the main home; no force acts before the
          // next rebuild, which streams it with the outside particles
          d.p.cell[idx] = cell;
          d.p.ox[idx] = ox; d.p.oy[idx] = oy; d.p.oz[idx] = oz;
          d.p.vx[idx] = vx; d.p.vy[idx] = vy; d.p.vz[idx] = vz;
          d.p.flag[idx] = (uint8_t)((fl & FLAG_SPECIES) | FLAG_PASSIVE);
          continue;
        }
        stream_one(kp, d.react_box, cell, ox, oy, oz, vx, vy, vz, fl, false, 1);
        const T msd = msd_now + (vx * vx + vy * vy + vz * vz) * (kp.dt * kp.dt);
        msdmax = msd > msdmax ? msd : msdmax;
        cg::coalesced_group g = cg::coalesced_threads();
        unsigned int bslot = 0;
        if (g.thread_rank() == 0) bslot = atomicAdd(&d.ctr->n_inside_new, g.size());
        bslot = g.shfl(bslot, 0);
        const unsigned int k = bslot + g.thread_rank();
        if ((int64_t)k >= d.sh2.cap) { atomicOr(&d.ctr->status, DEV_ERR_SHELL_OVERFLOW); continue; }
        d.sh2.idx[k] = idx;
        d.sh2.mid[k] = d.sh.mid[j];
        d.sh2.cell[k] = cell;
        d.sh2.ox[k] = ox; d.sh2.oy[k] = oy; d.sh2.oz[k] = oz;
        d.sh2.vx[k] = vx; d.sh2.vy[k] = vy; d.sh2.vz[k] = vz;
        d.sh2.msd[k] = msd;
        d.sh2.flag[k] = fl;
        d.sh2.nonbulk[k] = d.sh.nonbulk[j];
        d.sh2.np[k] = (uint8_t)np;
        *reinterpret_cast<uint4*>(d.sh2.sph + (size_t)k * PAIRMAX) = packed;
        d.p.cell[idx] = k;
        continue;
      }
      stream_one(kp, d.react_box, cell, ox, oy, oz, vx, vy, vz, fl, false, 1);
      T msd = d.sh.msd[j] + (vx * vx + vy * vy + vz * vz) * (kp.dt * kp.dt);
      d.sh.msd[j] = msd;
      msdmax = msd > msdmax ? msd : msdmax;
      d.sh.cell[j] = cell;
      d.sh.ox[j] = ox; d.sh.oy[j] = oy; d.sh.oz[j] = oz;
      d.sh.flag[j] = fl;
    }
    if (a.watch_build) watch_append(&d.ctr->n_watch, d.watch, d.sh.idx[j]);
    d.sh.vx[j] = vx; d.sh.vy[j] = vy; d.sh.vz[j] = vz;
  }
  if (a.advance) block_max_to<T>(&d.ctr->maxmsd[(a.step + 1) & 1], msdmax);
}

// Publish the shell packed by k_shell_advance.
template <typename T>
__global__ void k_shell_commit(Counters* c, int64_t cap) {
  unsigned int m = c->n_inside_new;
  if ((int64_t)m > cap) m = (unsigned int)cap;
  c->n_inside = m;
  c->n_inside_new = 0u;
}

template <typename T>
void Launch<T>::advance(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st) {
  k_shell_advance<T><<<a.g_shell > 0 ? a.g_shell : a.grid, TPB, 0, st>>>(d, kp, a, 0);
  LAUNCH_COUNT();
  if (a.advance && a.horizon > 0) {
    k_shell_commit<T><<<1, 1, 0, st>>>(d.ctr, d.sh2.cap);
    LAUNCH_COUNT();
  }
}

template <typename T>
void Launch<T>::rotate_shell(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st) {
  k_shell_advance<T><<<a.g_shell > 0 ? a.g_shell : a.grid, TPB, 0, st>>>(d, kp, a, 1);
  LAUNCH_COUNT();
  if (a.advance && a.horizon > 0) {
    k_shell_commit<T><<<1, 1, 0, st>>>(d.ctr, d.sh2.cap);
    LAUNCH_COUNT();
  }
}

// ------------------------------------------------------- shell ordering ----
// Counting sort of the shell entries by (first sphere, pair class): the
// entries a warp processes then mostly share their spheres and their pair
// count, so the per-sphere warp reductions of k_force run once or twice per
// warp instead of once per sphere present, and a warp of single-pair entries
// does not loop over second pairs.  Classes: 0 one pair, 1 the second pair is
// the first sphere's dimer partner, 2 any other second pair.  The order
// within a bucket is not specified (results do not depend on it beyond the
// summation order of the FP64 sphere-force atomics).
__device__ __forceinline__ int shell_bucket(uint32_t s01, int np) {
  const int s0 = (int)(s01 & 0xFFFFu), s1 = (int)(s01 >> 16);
  const int cls = np <= 1 ? 0 : (s1 == (s0 ^ 1) ? 1 : 2);
  return s0 * SHELL_CLASSES + cls;
}
template <typename T>
__global__ void k_shell_hist(Dev<T> d, KParams<T> kp) {
  if (d.ctr->abort_step) return;
  const unsigned int nin = d.ctr->n_inside;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); base < (int64_t)nin; base += stride) {
    const int64_t j = base + lane;
    int s = -1;
    if (j < (int64_t)nin) {
      const uint32_t s01 = *reinterpret_cast<const uint32_t*>(d.sh2.sph + (size_t)j * PAIRMAX);
      s = (int)(s01 & 0xFFFFu) < kp.ns ? shell_bucket(s01, d.sh2.np[j]) : -1;
      if (!chk(s >= 0, d.ctr, 123, s01)) s = -1;
    }
    // one atomic per bucket present in the warp
    const unsigned peers = __match_any_sync(0xffffffffu, s);
    if (s >= 0 && lane == __ffs(peers) - 1) atomicAdd(&d.sph_cnt[s], (unsigned)__popc(peers));
  }
}

template <typename T>
__global__ void k_shell_scan(Dev<T> d, KParams<T> kp) {
  if (d.ctr->abort_step) return;
  // one block: exclusive scan of the ns counts, which become the cursors
  __shared__ uint32_t part[TPB];
  const int nbk = kp.ns * SHELL_CLASSES;
  const int per = (nbk + TPB - 1) / TPB;
  const int lo = threadIdx.x * per, hi = min(lo + per, nbk);
  uint32_t sum = 0;
  for (int s = lo; s < hi; ++s) sum += d.sph_cnt[s];
  part[threadIdx.x] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int t = 0; t < TPB; ++t) { const uint32_t v = part[t]; part[t] = run; run += v; }
  }
  __syncthreads();
  uint32_t run = part[threadIdx.x];
  for (int s = lo; s < hi; ++s) { const uint32_t v = d.sph_cnt[s]; d.sph_base[s] = run; d.sph_cnt[s] = 0; run += v; }
}

template <typename T>
__global__ void k_shell_scatter(Dev<T> d, KParams<T> kp) {
  if (d.ctr->abort_step) return;
  const unsigned int nin = d.ctr->n_inside;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); base < (int64_t)nin; base += stride) {
    const int64_t j = base + lane;
    uint4 packed = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
    int s = -1;
    if (j < (int64_t)nin) {
      packed = *reinterpret_cast<const uint4*>(d.sh2.sph + (size_t)j * PAIRMAX);
      s = (int)(packed.x & 0xFFFFu) < kp.ns ? shell_bucket(packed.x, d.sh2.np[j]) : -1;
      if (!chk(s >= 0, d.ctr, 124, packed.x)) s = -1;
    }
    // one atomic per bucket present in the warp; its lanes take consecutive slots
    const unsigned peers = __match_any_sync(0xffffffffu, s);
    const int lead = __ffs(peers) - 1;
    uint32_t first = 0;
    if (s >= 0 && lane == lead) first = atomicAdd(&d.sph_cnt[s], (unsigned)__popc(peers));
    first = __shfl_sync(0xffffffffu, first, lead);
    if (s < 0) continue;
    const uint32_t k = d.sph_base[s] + first + __popc(peers & ((1u << lane) - 1u));
    if (!chk((int64_t)k < d.sh.cap, d.ctr, 125, k)) continue;
    const uint32_t idx = d.sh2.idx[j];
    d.sh.idx[k] = idx;
    d.sh.mid[k] = d.sh2.mid[j];
    d.sh.cell[k] = d.sh2.cell[j];
    d.sh.ox[k] = d.sh2.ox[j]; d.sh.oy[k] = d.sh2.oy[j]; d.sh.oz[k] = d.sh2.oz[j];
    d.sh.vx[k] = d.sh2.vx[j]; d.sh.vy[k] = d.sh2.vy[j]; d.sh.vz[k] = d.sh2.vz[j];
    d.sh.msd[k] = d.sh2.msd[j];
    d.sh.flag[k] = d.sh2.flag[j];
    d.sh.nonbulk[k] = d.sh2.nonbulk[j];
    d.sh.np[k] = d.sh2.np[j];
    *reinterpret_cast<uint4*>(d.sh.sph + (size_t)k * PAIRMAX) = packed;
    d.p.cell[idx] = k;
  }
}

template <typename T>
__global__ void k_shell_clear_counts(Dev<T> d, KParams<T> kp) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < kp.ns * SHELL_CLASSES; s += gridDim.x * blockDim.x)
    d.sph_cnt[s] = 0u;
}

template <typename T>
void Launch<T>::sort_shell(const Dev<T>& d, const KParams<T>& kp, cudaStream_t st) {
  if (kp.ns == 0) return;
  k_shell_clear_counts<T><<<(kp.ns * SHELL_CLASSES + TPB - 1) / TPB, TPB, 0, st>>>(d, kp);
  k_shell_hist<T><<<1024, TPB, 0, st>>>(d, kp);
  k_shell_scan<T><<<1, TPB, 0, st>>>(d, kp);
  k_shell_scatter<T><<<1024, TPB, 0, st>>>(d, kp);
  LAUNCH_COUNT(); LAUNCH_COUNT(); LAUNCH_COUNT(); LAUNCH_COUNT();
}

// ---------------------------------------------------------------- dimers ----
// forces_mod.f95:273-335 as called at evolve_mod.f95:597,600 (the actual
// arguments 3R^3 and 9R^9 bind to the dummies named r9R9 and r3R3).
template <typename T>
__device__ void lj_wall(const KParams<T>& kp, double zdim, double RwR, double w3, double& fz, double& pot) {
  const double cutoff2 = (RwR * w3) * (RwR * w3);
  const double R3 = RwR * RwR * RwR, R9 = R3 * R3 * R3;
  const double r9R9 = 3.0 * R3, r3R3 = 9.0 * R9;
  const double pref = 0.5 * 3. * sqrt(3.0);
  double dR = kp.Ld[2] - zdim;
  if (dR * dR < cutoff2) {
    double IdRsq = 1. / (dR * dR);
    double IdR3 = pow(IdRsq, 1.5);
    double IdR9 = IdR3 * IdR3 * IdR3, IdR5 = IdR3 * IdRsq, IdR11 = IdR9 * IdRsq;
    double Fb = pref * kp.ew * (r9R9 * IdR11 - r3R3 * IdR5);
    fz = Fb * dR;
    pot = pref * kp.ew * (R9 * IdR9 - R3 * IdR3) + 1.0;
  }
  dR = 0. - zdim;
  if (dR * dR < cutoff2) {
    double IdRsq = 1. / (dR * dR);
    double IdR3 = pow(IdRsq, 1.5);
    double IdR9 = IdR3 * IdR3 * IdR3, IdR5 = IdR3 * IdRsq, IdR11 = IdR9 * IdRsq;
    double Fb = pref * kp.ew * (r9R9 * IdR11 - r3R3 * IdR5);
    fz = fz + Fb * dR;
    pot = pot + pref * kp.ew * (R9 * IdR9 - R3 * IdR3) + 1.0;
  }
}

__device__ __forceinline__ double dmin_image(double d, double L) {
  if (d > 0.5 * L) d -= L;
  else if (d < -0.5 * L) d += L;
  return d;
}

// One thread per dimer (evolve_mod.f95:605-636 totals, :679-724 RATTLE
// velocities, :320-417 RATTLE positions of the next step), on register copies
// of the dimer state.  mode bit 0: finish the force step (totals +
// RATTLE-v); bit 1: RATTLE-x.  The FP64 parity build performs the reference's
// operation sequence; the FP32 production build multiplies by precomputed
// reciprocals and wraps the positions once after the RATTLE-x iterations (the
// constraint uses minimum-image separations, so the in-loop wraps of the
// reference only change the stored result, which the final wrap reproduces).
template <typename T>
__global__ void k_dimer(Dev<T> d, KParams<T> kp, StepArgs a, int mode, double w3, int rattle_max) {
  if (d.ctr->abort_step) return;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kp.nd) return;
  constexpr bool fast = sizeof(T) == 4;
  const double dt = kp.dtd, Mc = kp.mc, Mn = kp.mn, Dcn = kp.dcn;
  const double hIMc = kp.hIMc, hIMn = kp.hIMn, IIM = kp.IIM;
  const double iMc = kp.iMc, iMn = kp.iMn, iD2 = kp.iD2, iMcdt = kp.iMcdt, iMndt = kp.iMndt;
  const bool per = kp.geometry == 1;
  const int nwrap = per ? 3 : 2;
  const int s1 = 2 * k, s2 = 2 * k + 1;
  double X1[3], X2[3], V1[3], V2[3], F1[3], F2[3], Q1[3], Q2[3];
  for (int c = 0; c < 3; ++c) {
    X1[c] = d.dpos[3 * s1 + c]; X2[c] = d.dpos[3 * s2 + c];
    V1[c] = d.dvel[3 * s1 + c]; V2[c] = d.dvel[3 * s2 + c];
    F1[c] = d.dfrc[3 * s1 + c]; F2[c] = d.dfrc[3 * s2 + c];
    Q1[c] = d.dq[3 * s1 + c]; Q2[c] = d.dq[3 * s2 + c];
  }
  unsigned long long iters = 0;
  if (mode & 1) {
    double pot = 0.;
    for (int i = 0; i < 2; ++i) {
      const int s = 2 * k + i;
      double* F = i == 0 ? F1 : F2;
      double fw = 0., pw = 0.;
      if (!per) lj_wall(kp, (i == 0 ? X1 : X2)[2], i == 0 ? kp.rwc : kp.rwn, w3, fw, pw);
      F[0] = d.facc[4 * s + 0] + d.fmot[4 * s + 0];
      F[1] = d.facc[4 * s + 1] + d.fmot[4 * s + 1];
      F[2] = d.facc[4 * s + 2] + d.fmot[4 * s + 2] + fw;
      pot += d.facc[4 * s + 3] + d.fmot[4 * s + 3] + pw;
      d.facc[4 * s + 0] = 0.; d.facc[4 * s + 1] = 0.; d.facc[4 * s + 2] = 0.; d.facc[4 * s + 3] = 0.;
    }
    d.dpot[k] = pot;
    for (int c = 0; c < 3; ++c) { V1[c] = Q1[c] + hIMc * F1[c]; V2[c] = Q2[c] + hIMn * F2[c]; }
    int acc = 0;
    for (;;) {
      double dV[3], dd[3];
      for (int c = 0; c < 3; ++c) { dV[c] = V1[c] - V2[c]; dd[c] = X1[c] - X2[c]; }
      dd[0] = dmin_image(dd[0], kp.Ld[0]);
      dd[1] = dmin_image(dd[1], kp.Ld[1]);
      if (per) dd[2] = dmin_image(dd[2], kp.Ld[2]);
      double Con2diff = 2.0 * (dV[0] * dd[0] + dV[1] * dd[1] + dV[2] * dd[2]);
      if (fabs(Con2diff) < 1.e-8) break;
      if (acc == rattle_max) { atomicOr(&d.ctr->status, DEV_ERR_RATTLE); break; }
      if (fast) {
        const double O2 = -(0.5 * (IIM * Con2diff) * iD2);
        for (int c = 0; c < 3; ++c) {
          V1[c] = V1[c] + O2 * dd[c] * iMc;
          V2[c] = V2[c] - O2 * dd[c] * iMn;
        }
      } else {
        double O = -(0.25 * (IIM * Con2diff) / (Dcn * Dcn));
        for (int c = 0; c < 3; ++c) {
          V1[c] = V1[c] + 2.0 * O * dd[c] / Mc;
          V2[c] = V2[c] - 2.0 * O * dd[c] / Mn;
        }
      }
      acc++;
    }
    iters += acc;
    for (int c = 0; c < 3; ++c) {
      d.dvel[3 * s1 + c] = V1[c]; d.dvel[3 * s2 + c] = V2[c];
      d.dfrc[3 * s1 + c] = F1[c]; d.dfrc[3 * s2 + c] = F2[c];
    }
  }
  if (mode & 2) {
    double pr1[3], pr2[3], dP[3];
    for (int c = 0; c < 3; ++c) { pr1[c] = X1[c]; pr2[c] = X2[c]; dP[c] = X1[c] - X2[c]; }
    dP[0] = dmin_image(dP[0], kp.Ld[0]);
    dP[1] = dmin_image(dP[1], kp.Ld[1]);
    if (per) dP[2] = dmin_image(dP[2], kp.Ld[2]);
    for (int c = 0; c < 3; ++c) { Q1[c] = V1[c] + hIMc * F1[c]; Q2[c] = V2[c] + hIMn * F2[c]; }
    for (int c = 0; c < 3; ++c) { X1[c] = X1[c] + dt * Q1[c]; X2[c] = X2[c] + dt * Q2[c]; }
    if (!fast) {
      for (int c = 0; c < nwrap; ++c) {
        X1[c] = X1[c] - kp.Ld[c] * floor(X1[c] / kp.Ld[c]);
        X2[c] = X2[c] - kp.Ld[c] * floor(X2[c] / kp.Ld[c]);
      }
    }
    int acc = 0;
    for (;;) {
      double dd[3];
      for (int c = 0; c < 3; ++c) dd[c] = X1[c] - X2[c];
      dd[0] = dmin_image(dd[0], kp.Ld[0]);
      dd[1] = dmin_image(dd[1], kp.Ld[1]);
      if (per) dd[2] = dmin_image(dd[2], kp.Ld[2]);
      double Con1diff = (dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]) - Dcn * Dcn;
      if (fabs(Con1diff) < 1.e-6) break;
      if (acc == rattle_max) { atomicOr(&d.ctr->status, DEV_ERR_RATTLE); break; }
      const double den = dd[0] * dP[0] + dd[1] * dP[1] + dd[2] * dP[2];
      double G;
      if (fast) {
        // the iteration converges to the tolerance whatever the last bits of
        // G are: a float reciprocal refined twice replaces the division
        double r = (double)__frcp_rn((float)den);
        r = r * (2.0 - den * r);
        r = r * (2.0 - den * r);
        G = -(0.25 * Con1diff * IIM) * r;
      } else {
        G = -(0.25 * Con1diff * IIM / den);
      }
      if (fast) {
        const double G2 = 2.0 * G;
        for (int c = 0; c < 3; ++c) {
          X1[c] = pr1[c] + Q1[c] * dt + G2 * dP[c] * iMc;
          X2[c] = pr2[c] + Q2[c] * dt - G2 * dP[c] * iMn;
          Q1[c] = Q1[c] + G2 * dP[c] * iMcdt;
          Q2[c] = Q2[c] - G2 * dP[c] * iMndt;
        }
      } else {
        for (int c = 0; c < 3; ++c) {
          X1[c] = pr1[c] + Q1[c] * dt + 2.0 * G * dP[c] / Mc;
          X2[c] = pr2[c] + Q2[c] * dt - 2.0 * G * dP[c] / Mn;
        }
        for (int c = 0; c < nwrap; ++c) {
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
    if (fast) {
      // one step moves a sphere far less than a box edge: a single shift
      for (int c = 0; c < nwrap; ++c) {
        const double L = kp.Ld[c];
        if (X1[c] >= L) X1[c] -= L; else if (X1[c] < 0.0) X1[c] += L;
        if (X2[c] >= L) X2[c] -= L; else if (X2[c] < 0.0) X2[c] += L;
        if (!(X1[c] >= 0.0 && X1[c] < L)) X1[c] = X1[c] - L * floor(X1[c] / L);
        if (!(X2[c] >= 0.0 && X2[c] < L)) X2[c] = X2[c] - L * floor(X2[c] / L);
      }
    }
    iters += acc;
    for (int c = 0; c < 3; ++c) {
      d.dpos[3 * s1 + c] = X1[c]; d.dpos[3 * s2 + c] = X2[c];
      d.dq[3 * s1 + c] = Q1[c]; d.dq[3 * s2 + c] = Q2[c];
    }
    for (int i = 0; i < 2; ++i) {
      const double* X = i == 0 ? X1 : X2;
      const double fx = floor(X[0]), fy = floor(X[1]), fz = floor(X[2]);
      SphereRel<T> r;
      r.cx = (int)fx; r.cy = (int)fy; r.cz = (int)fz;
      r.ox = (T)(X[0] - fx); r.oy = (T)(X[1] - fy); r.oz = (T)(X[2] - fz);
      d.srel[2 * k + i] = r;
    }
  }
  if (iters) atomicAdd(&d.ctr->rattle_iters, iters);
}

// rotational_code/2d_array/forces_mod.f95:177-201: harmonic z tether.
__device__ __forceinline__ void harmonic_tether(const double zdim, const double zdimeq, const double k_harm,
                                                double& f, double& pot) {
  const double zdiff = zdim - zdimeq;
  f = -1. * k_harm * zdiff;
  pot = 0.5 * k_harm * (zdiff * zdiff);
}

// One thread per anchored rotor (rotational_code/2d_array/evolve_mod.f95:
// 533-557 totals with the tether, :596-650 RATTLE velocities, :283-391
// RATTLE positions), in the reference's FP64 operation sequence in both
// builds (a handful of rotors per run).  Besides the bond, the positions hold
// the midpoint 0.5 (X1 + X2) (wrapped into the box in x and y) at the anchor,
// with the correction H = -4 IIM (midpoint - anchor) applied as H / (2 M) to
// each sphere, and the velocities hold the midpoint velocity at zero.
template <typename T>
__global__ void k_rotor(Dev<T> d, KParams<T> kp, StepArgs a, int mode, int rattle_max) {
  if (d.ctr->abort_step) return;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kp.nd) return;
  const double dt = kp.dtd, Mc = kp.mc, Mn = kp.mn, Dcn = kp.dcn;
  const double hIMc = kp.hIMc, hIMn = kp.hIMn, IIM = kp.IIM;
  // the FP32 build multiplies by precomputed reciprocals where the reference
  // divides (FP64 divisions dominate the iteration chain on this part); the
  // FP64 parity build keeps the reference's operation sequence
  constexpr bool fast = sizeof(T) == 4;
  const double iMc = kp.iMc, iMn = kp.iMn, iD2 = kp.iD2, iMcdt = kp.iMcdt, iMndt = kp.iMndt;
  const bool per = kp.geometry == 1;
  const int nwrap = per ? 3 : 2;
  const int s1 = 2 * k, s2 = 2 * k + 1;
  double X1[3], X2[3], V1[3], V2[3], F1[3], F2[3], Q1[3], Q2[3], A[3];
  for (int c = 0; c < 3; ++c) {
    X1[c] = d.dpos[3 * s1 + c]; X2[c] = d.dpos[3 * s2 + c];
    V1[c] = d.dvel[3 * s1 + c]; V2[c] = d.dvel[3 * s2 + c];
    F1[c] = d.dfrc[3 * s1 + c]; F2[c] = d.dfrc[3 * s2 + c];
    Q1[c] = d.dq[3 * s1 + c]; Q2[c] = d.dq[3 * s2 + c];
    A[c] = d.anchor[3 * k + c];
  }
  unsigned long long iters = 0;
  if (mode & 1) {
    double pot = 0.;
    for (int i = 0; i < 2; ++i) {
      const int s = 2 * k + i;
      double* F = i == 0 ? F1 : F2;
      double fw = 0., pw = 0.;
      harmonic_tether((i == 0 ? X1 : X2)[2], kp.tether_z, kp.tether_k, fw, pw);
      F[0] = d.facc[4 * s + 0];
      F[1] = d.facc[4 * s + 1];
      F[2] = d.facc[4 * s + 2] + fw;
      pot += d.facc[4 * s + 3] + pw;
      d.facc[4 * s + 0] = 0.; d.facc[4 * s + 1] = 0.; d.facc[4 * s + 2] = 0.; d.facc[4 * s + 3] = 0.;
    }
    d.dpot[k] = pot;
    for (int c = 0; c < 3; ++c) { V1[c] = Q1[c] + hIMc * F1[c]; V2[c] = Q2[c] + hIMn * F2[c]; }
    int acc = 0;
    for (;;) {
      double dV[3], dd[3], Vm[3];
      for (int c = 0; c < 3; ++c) { dV[c] = V1[c] - V2[c]; dd[c] = X1[c] - X2[c]; }
      dd[0] = dmin_image(dd[0], kp.Ld[0]);
      dd[1] = dmin_image(dd[1], kp.Ld[1]);
      if (per) dd[2] = dmin_image(dd[2], kp.Ld[2]);
      const double Con2diff = dV[0] * dd[0] + dV[1] * dd[1] + dV[2] * dd[2];
      for (int c = 0; c < 3; ++c) Vm[c] = 0.5 * (V1[c] + V2[c]);
      if (fabs(Con2diff) < 1.e-8 && fabs(Vm[0]) < 1.e-8 && fabs(Vm[1]) < 1.e-8 && fabs(Vm[2]) < 1.e-8) break;
      if (acc == rattle_max) { atomicOr(&d.ctr->status, DEV_ERR_RATTLE); break; }
      if (fast) {
        const double O = -(0.25 * (IIM * Con2diff) * iD2);
        for (int c = 0; c < 3; ++c) {
          const double hP = -(2.0 * Vm[c] * IIM);
          V1[c] = V1[c] + (O * dd[c] + hP) * iMc;
          V2[c] = V2[c] + (hP - O * dd[c]) * iMn;
        }
      } else {
        const double O = -(0.25 * (IIM * Con2diff) / (Dcn * Dcn));
        for (int c = 0; c < 3; ++c) {
          const double P = -(4.0 * Vm[c] * IIM);
          V1[c] = V1[c] + O * dd[c] / Mc + 0.5 * P / Mc;
          V2[c] = V2[c] - O * dd[c] / Mn + 0.5 * P / Mn;
        }
      }
      acc++;
    }
    iters += acc;
    for (int c = 0; c < 3; ++c) {
      d.dvel[3 * s1 + c] = V1[c]; d.dvel[3 * s2 + c] = V2[c];
      d.dfrc[3 * s1 + c] = F1[c]; d.dfrc[3 * s2 + c] = F2[c];
    }
  }
  if (mode & 2) {
    double pr1[3], pr2[3], dP[3];
    for (int c = 0; c < 3; ++c) { pr1[c] = X1[c]; pr2[c] = X2[c]; dP[c] = X1[c] - X2[c]; }
    dP[0] = dmin_image(dP[0], kp.Ld[0]);
    dP[1] = dmin_image(dP[1], kp.Ld[1]);
    if (per) dP[2] = dmin_image(dP[2], kp.Ld[2]);
    for (int c = 0; c < 3; ++c) { Q1[c] = V1[c] + hIMc * F1[c]; Q2[c] = V2[c] + hIMn * F2[c]; }
    for (int c = 0; c < 3; ++c) { X1[c] = X1[c] + dt * Q1[c]; X2[c] = X2[c] + dt * Q2[c]; }
    for (int c = 0; c < nwrap; ++c) {
      X1[c] = X1[c] - kp.Ld[c] * floor(X1[c] / kp.Ld[c]);
      X2[c] = X2[c] - kp.Ld[c] * floor(X2[c] / kp.Ld[c]);
    }
    int acc = 0;
    for (;;) {
      double dd[3], D[3];
      for (int c = 0; c < 3; ++c) dd[c] = X1[c] - X2[c];
      dd[0] = dmin_image(dd[0], kp.Ld[0]);
      dd[1] = dmin_image(dd[1], kp.Ld[1]);
      if (per) dd[2] = dmin_image(dd[2], kp.Ld[2]);
      for (int c = 0; c < 3; ++c) {
        double m = 0.5 * (X1[c] + X2[c]);
        if (c < 2) {
          if (m >= kp.Ld[c]) m = m - kp.Ld[c];
          else if (m < 0.) m = m + kp.Ld[c];
        }
        D[c] = m - A[c];
      }
      const double Con1diff = (dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]) - Dcn * Dcn;
      if (fabs(Con1diff) < 1.e-6 && fabs(D[0]) < 1.e-6 && fabs(D[1]) < 1.e-6 && fabs(D[2]) < 1.e-6) break;
      if (acc == rattle_max) { atomicOr(&d.ctr->status, DEV_ERR_RATTLE); break; }
      const double den = dd[0] * dP[0] + dd[1] * dP[1] + dd[2] * dP[2];
      if (fast) {
        // a float reciprocal refined twice replaces the division (the
        // iteration converges to the tolerance whatever G's last bits are)
        double r = (double)__frcp_rn((float)den);
        r = r * (2.0 - den * r);
        r = r * (2.0 - den * r);
        const double G = -(0.25 * Con1diff * IIM) * r;
        for (int c = 0; c < 3; ++c) {
          const double hH = -(2.0 * IIM * D[c]);
          const double u1 = G * dP[c] + hH, u2 = hH - G * dP[c];
          X1[c] = pr1[c] + Q1[c] * dt + u1 * iMc;
          X2[c] = pr2[c] + Q2[c] * dt + u2 * iMn;
          const double L = kp.Ld[c];
          if (X1[c] >= L) X1[c] -= L; else if (X1[c] < 0.0) X1[c] += L;
          if (X2[c] >= L) X2[c] -= L; else if (X2[c] < 0.0) X2[c] += L;
          Q1[c] = Q1[c] + u1 * iMcdt;
          Q2[c] = Q2[c] + u2 * iMndt;
        }
      } else {
        const double G = -(0.25 * Con1diff * IIM / den);
        double H[3];
        for (int c = 0; c < 3; ++c) H[c] = -(4.0 * IIM * D[c]);
        for (int c = 0; c < 3; ++c) {
          X1[c] = pr1[c] + Q1[c] * dt + G * dP[c] / Mc + 0.5 * H[c] / Mc;
          X2[c] = pr2[c] + Q2[c] * dt - G * dP[c] / Mn + 0.5 * H[c] / Mn;
        }
        for (int c = 0; c < 3; ++c) {
          X1[c] = X1[c] - kp.Ld[c] * floor(X1[c] / kp.Ld[c]);
          X2[c] = X2[c] - kp.Ld[c] * floor(X2[c] / kp.Ld[c]);
        }
        for (int c = 0; c < 3; ++c) {
          Q1[c] = Q1[c] + G * dP[c] / (Mc * dt) + 0.5 * H[c] / (Mc * dt);
          Q2[c] = Q2[c] - G * dP[c] / (Mn * dt) + 0.5 * H[c] / (Mn * dt);
        }
      }
      acc++;
    }
    iters += acc;
    for (int c = 0; c < 3; ++c) {
      d.dpos[3 * s1 + c] = X1[c]; d.dpos[3 * s2 + c] = X2[c];
      d.dq[3 * s1 + c] = Q1[c]; d.dq[3 * s2 + c] = Q2[c];
    }
    for (int i = 0; i < 2; ++i) {
      const double* X = i == 0 ? X1 : X2;
      const double fx = floor(X[0]), fy = floor(X[1]), fz = floor(X[2]);
      SphereRel<T> r;
      r.cx = (int)fx; r.cy = (int)fy; r.cz = (int)fz;
      r.ox = (T)(X[0] - fx); r.oy = (T)(X[1] - fy); r.oz = (T)(X[2] - fz);
      d.srel[2 * k + i] = r;
    }
  }
  if (iters) atomicAdd(&d.ctr->rattle_iters, iters);
}

// Sum over the four lanes of a dimer's group (mask: those lanes, which
// always take the same branches); every lane gets the same bits (the
// butterfly adds the same pairs in every lane).
__device__ __forceinline__ double group4_sum(unsigned mask, double v) {
  v += __shfl_xor_sync(mask, v, 1);
  v += __shfl_xor_sync(mask, v, 2);
  return v;
}

// The FP32 build's dimer step with the three Cartesian components of a dimer
// on three lanes of a 4-lane group (the fourth holds zeros and the energy):
// the same update as k_dimer's fast path (totals, RATTLE velocities, RATTLE
// positions, single-shift wrap), with the constraint dot products summed
// across the group.  On this part FP64 instructions are issued at a few lanes
// per SM cycle, so the per-dimer chain of FP64 instructions, not the lane
// count, sets the time; splitting the components shortens that chain about
// threefold.  The FP64 parity build keeps k_dimer and the oracle's order.
template <typename T>
__global__ void k_dimer_split(Dev<T> d, KParams<T> kp, StepArgs a, int mode, double w3, int rattle_max) {
  if (d.ctr->abort_step) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = t >> 2, c = t & 3;
  const unsigned gmask = 0xFu << (threadIdx.x & 28);   // this group's four lanes
  const bool live = k < kp.nd;        // the whole 4-lane group agrees
  const int kk = live ? k : 0;
  const bool comp = c < 3;
  const double dt = kp.dtd, Dcn = kp.dcn;
  const double hIMc = kp.hIMc, hIMn = kp.hIMn, IIM = kp.IIM;
  const double iMc = kp.iMc, iMn = kp.iMn, iD2 = kp.iD2, iMcdt = kp.iMcdt, iMndt = kp.iMndt;
  const bool per = kp.geometry == 1;
  const int cc = comp ? c : 0;
  const bool wrapc = comp && (c < 2 || per);
  const double L = kp.Ld[cc];
  const int s1 = 2 * kk, s2 = 2 * kk + 1;
  double X1 = 0, X2 = 0, V1 = 0, V2 = 0, F1 = 0, F2 = 0, Q1 = 0, Q2 = 0;
  if (live && comp) {
    X1 = d.dpos[3 * s1 + c]; X2 = d.dpos[3 * s2 + c];
    V1 = d.dvel[3 * s1 + c]; V2 = d.dvel[3 * s2 + c];
    F1 = d.dfrc[3 * s1 + c]; F2 = d.dfrc[3 * s2 + c];
    Q1 = d.dq[3 * s1 + c]; Q2 = d.dq[3 * s2 + c];
  }
  unsigned long long iters = 0;
  if (mode & 1) {
    double fw1 = 0., pw1 = 0., fw2 = 0., pw2 = 0.;
    if (live && c == 2 && !per) {
      lj_wall(kp, X1, kp.rwc, w3, fw1, pw1);
      lj_wall(kp, X2, kp.rwn, w3, fw2, pw2);
    }
    // the wall energies travel from the z lane to the energy lane
    const int zl = (threadIdx.x & 31 & ~3) | 2;
    const double p1 = __shfl_sync(gmask, pw1, zl), p2 = __shfl_sync(gmask, pw2, zl);
    if (live) {
      const int q = comp ? c : 3;
      const double a1 = d.facc[4 * s1 + q] + d.fmot[4 * s1 + q];
      const double a2 = d.facc[4 * s2 + q] + d.fmot[4 * s2 + q];
      d.facc[4 * s1 + q] = 0.; d.facc[4 * s2 + q] = 0.;
      if (comp) {
        F1 = a1 + (c == 2 ? fw1 : 0.);
        F2 = a2 + (c == 2 ? fw2 : 0.);
      } else {
        d.dpot[kk] = (a1 + p1) + (a2 + p2);
      }
    }
    if (comp) { V1 = Q1 + hIMc * F1; V2 = Q2 + hIMn * F2; }
    int acc = 0;
    for (;;) {
      double dd = X1 - X2;
      if (wrapc) dd = dmin_image(dd, L);
      const double Con2diff = 2.0 * group4_sum(gmask, (V1 - V2) * dd);
      if (!live || fabs(Con2diff) < 1.e-8) break;
      if (acc == rattle_max) { if (c == 0) atomicOr(&d.ctr->status, DEV_ERR_RATTLE); break; }
      const double O2 = -(0.5 * (IIM * Con2diff) * iD2);
      V1 = V1 + O2 * dd * iMc;
      V2 = V2 - O2 * dd * iMn;
      acc++;
    }
    iters += acc;
    if (live && comp) {
      d.dvel[3 * s1 + c] = V1; d.dvel[3 * s2 + c] = V2;
      d.dfrc[3 * s1 + c] = F1; d.dfrc[3 * s2 + c] = F2;
    }
  }
  if (mode & 2) {
    const double pr1 = X1, pr2 = X2;
    double dP = X1 - X2;
    if (wrapc) dP = dmin_image(dP, L);
    if (!comp) dP = 0.;
    Q1 = V1 + hIMc * F1; Q2 = V2 + hIMn * F2;
    X1 = X1 + dt * Q1; X2 = X2 + dt * Q2;
    int acc = 0;
    for (;;) {
      double dd = X1 - X2;
      if (wrapc) dd = dmin_image(dd, L);
      if (!comp) dd = 0.;
      const double Con1diff = group4_sum(gmask, dd * dd) - Dcn * Dcn;
      if (!live || fabs(Con1diff) < 1.e-6) break;
      if (acc == rattle_max) { if (c == 0) atomicOr(&d.ctr->status, DEV_ERR_RATTLE); break; }
      const double den = group4_sum(gmask, dd * dP);
      double r = (double)__frcp_rn((float)den);
      r = r * (2.0 - den * r);
      r = r * (2.0 - den * r);
      const double G2 = 2.0 * (-(0.25 * Con1diff * IIM) * r);
      X1 = pr1 + Q1 * dt + G2 * dP * iMc;
      X2 = pr2 + Q2 * dt - G2 * dP * iMn;
      Q1 = Q1 + G2 * dP * iMcdt;
      Q2 = Q2 - G2 * dP * iMndt;
      acc++;
    }
    if (wrapc && (c < 2 || per)) {
      if (X1 >= L) X1 -= L; else if (X1 < 0.0) X1 += L;
      if (X2 >= L) X2 -= L; else if (X2 < 0.0) X2 += L;
      if (!(X1 >= 0.0 && X1 < L)) X1 = X1 - L * floor(X1 / L);
      if (!(X2 >= 0.0 && X2 < L)) X2 = X2 - L * floor(X2 / L);
    }
    iters += acc;
    if (live && comp) {
      d.dpos[3 * s1 + c] = X1; d.dpos[3 * s2 + c] = X2;
      d.dq[3 * s1 + c] = Q1; d.dq[3 * s2 + c] = Q2;
      const double f1 = floor(X1), f2 = floor(X2);
      SphereRel<T>& r1 = d.srel[s1];
      SphereRel<T>& r2 = d.srel[s2];
      if (c == 0) { r1.cx = (int)f1; r1.ox = (T)(X1 - f1); r2.cx = (int)f2; r2.ox = (T)(X2 - f2); }
      else if (c == 1) { r1.cy = (int)f1; r1.oy = (T)(X1 - f1); r2.cy = (int)f2; r2.oy = (T)(X2 - f2); }
      else { r1.cz = (int)f1; r1.oz = (T)(X1 - f1); r2.cz = (int)f2; r2.oz = (T)(X2 - f2); }
    }
  }
  if (live && c == 0 && iters) atomicAdd(&d.ctr->rattle_iters, iters);
}

// Sphere force totals and dimer potentials of a restart (restart_mod.f95:
// 505-528), one thread per dimer: the same sums as the first stage of
// k_dimer / k_dimer_split / k_rotor (pair sums, motor-motor forces, the wall
// or the rotor tether), with no RATTLE.
template <typename T>
__global__ void k_sphere_totals(Dev<T> d, KParams<T> kp, double w3) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kp.nd) return;
  const bool per = kp.geometry == 1;
  double pot = 0.;
  for (int i = 0; i < 2; ++i) {
    const int s = 2 * k + i;
    double fw = 0., pw = 0.;
    if (kp.rotor) harmonic_tether(d.dpos[3 * s + 2], kp.tether_z, kp.tether_k, fw, pw);
    else if (!per) lj_wall(kp, d.dpos[3 * s + 2], i == 0 ? kp.rwc : kp.rwn, w3, fw, pw);
    d.dfrc[3 * s + 0] = d.facc[4 * s + 0] + d.fmot[4 * s + 0];
    d.dfrc[3 * s + 1] = d.facc[4 * s + 1] + d.fmot[4 * s + 1];
    d.dfrc[3 * s + 2] = d.facc[4 * s + 2] + d.fmot[4 * s + 2] + fw;
    pot += d.facc[4 * s + 3] + d.fmot[4 * s + 3] + pw;
    d.facc[4 * s + 0] = 0.; d.facc[4 * s + 1] = 0.; d.facc[4 * s + 2] = 0.; d.facc[4 * s + 3] = 0.;
  }
  d.dpot[k] = pot;
}

template <typename T>
void Launch<T>::sphere_totals(const Dev<T>& d, const KParams<T>& kp, double w3, cudaStream_t st) {
  if (kp.nd == 0) return;
  k_sphere_totals<T><<<(kp.nd + 63) / 64, 64, 0, st>>>(d, kp, w3);
  LAUNCH_COUNT();
}

// The FP32 build's rotor step (k_rotor's fast path) with the three Cartesian
// components of a rotor on three lanes of a 4-lane group, the constraint dot
// products summed across the group and the convergence tests taken over it;
// the fourth lane holds zeros and the energy.  As for k_dimer_split, the
// per-rotor chain of FP64 instructions sets the time, and the split shortens
// it about threefold.
template <typename T>
__global__ void k_rotor_split(Dev<T> d, KParams<T> kp, StepArgs a, int mode, int rattle_max) {
  if (d.ctr->abort_step) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = t >> 2, c = t & 3;
  const unsigned gmask = 0xFu << (threadIdx.x & 28);   // this group's four lanes
  const bool live = k < kp.nd;        // the whole 4-lane group agrees
  const int kk = live ? k : 0;
  const bool comp = c < 3;
  const double dt = kp.dtd, Dcn = kp.dcn;
  const double hIMc = kp.hIMc, hIMn = kp.hIMn, IIM = kp.IIM;
  const double iMc = kp.iMc, iMn = kp.iMn, iD2 = kp.iD2, iMcdt = kp.iMcdt, iMndt = kp.iMndt;
  const bool per = kp.geometry == 1;
  const int cc = comp ? c : 0;
  const bool mi = comp && (c < 2 || per);   // minimum image on this axis
  const double L = kp.Ld[cc];
  const int s1 = 2 * kk, s2 = 2 * kk + 1;
  double X1 = 0, X2 = 0, V1 = 0, V2 = 0, F1 = 0, F2 = 0, Q1 = 0, Q2 = 0, A = 0;
  if (live && comp) {
    X1 = d.dpos[3 * s1 + c]; X2 = d.dpos[3 * s2 + c];
    V1 = d.dvel[3 * s1 + c]; V2 = d.dvel[3 * s2 + c];
    F1 = d.dfrc[3 * s1 + c]; F2 = d.dfrc[3 * s2 + c];
    Q1 = d.dq[3 * s1 + c]; Q2 = d.dq[3 * s2 + c];
    A = d.anchor[3 * kk + c];
  }
  unsigned long long iters = 0;
  if (mode & 1) {
    double fw1 = 0., pw1 = 0., fw2 = 0., pw2 = 0.;
    if (live && c == 2) {
      harmonic_tether(X1, kp.tether_z, kp.tether_k, fw1, pw1);
      harmonic_tether(X2, kp.tether_z, kp.tether_k, fw2, pw2);
    }
    // the tether energies travel from the z lane to the energy lane
    const int zl = (threadIdx.x & 31 & ~3) | 2;
    const double p1 = __shfl_sync(gmask, pw1, zl), p2 = __shfl_sync(gmask, pw2, zl);
    if (live) {
      const int q = comp ? c : 3;
      const double a1 = d.facc[4 * s1 + q], a2 = d.facc[4 * s2 + q];
      d.facc[4 * s1 + q] = 0.; d.facc[4 * s2 + q] = 0.;
      if (comp) {
        F1 = a1 + (c == 2 ? fw1 : 0.);
        F2 = a2 + (c == 2 ? fw2 : 0.);
      } else {
        d.dpot[kk] = (a1 + p1) + (a2 + p2);
      }
    }
    if (comp) { V1 = Q1 + hIMc * F1; V2 = Q2 + hIMn * F2; }
    int acc = 0;
    for (;;) {
      double dd = X1 - X2;
      if (mi) dd = dmin_image(dd, L);
      if (!comp) dd = 0.;
      const double Con2diff = group4_sum(gmask, (V1 - V2) * dd);
      const double Vm = 0.5 * (V1 + V2);
      const bool vm_ok = __all_sync(gmask, !comp || fabs(Vm) < 1.e-8);
      if (!live || (fabs(Con2diff) < 1.e-8 && vm_ok)) break;
      if (acc == rattle_max) { if (c == 0) atomicOr(&d.ctr->status, DEV_ERR_RATTLE); break; }
      const double O = -(0.25 * (IIM * Con2diff) * iD2);
      const double hP = -(2.0 * Vm * IIM);
      V1 = V1 + (O * dd + hP) * iMc;
      V2 = V2 + (hP - O * dd) * iMn;
      acc++;
    }
    iters += acc;
    if (live && comp) {
      d.dvel[3 * s1 + c] = V1; d.dvel[3 * s2 + c] = V2;
      d.dfrc[3 * s1 + c] = F1; d.dfrc[3 * s2 + c] = F2;
    }
  }
  if (mode & 2) {
    const double pr1 = X1, pr2 = X2;
    double dP = X1 - X2;
    if (mi) dP = dmin_image(dP, L);
    if (!comp) dP = 0.;
    Q1 = V1 + hIMc * F1; Q2 = V2 + hIMn * F2;
    X1 = X1 + dt * Q1; X2 = X2 + dt * Q2;
    if (comp && (c < 2 || per)) {
      if (X1 >= L) X1 -= L; else if (X1 < 0.0) X1 += L;
      if (X2 >= L) X2 -= L; else if (X2 < 0.0) X2 += L;
    }
    int acc = 0;
    for (;;) {
      double dd = X1 - X2;
      if (mi) dd = dmin_image(dd, L);
      if (!comp) dd = 0.;
      double m = 0.5 * (X1 + X2);
      if (c < 2) {
        if (m >= L) m = m - L;
        else if (m < 0.) m = m + L;
      }
      const double D = m - A;
      const double Con1diff = group4_sum(gmask, dd * dd) - Dcn * Dcn;
      const bool d_ok = __all_sync(gmask, !comp || fabs(D) < 1.e-6);
      if (!live || (fabs(Con1diff) < 1.e-6 && d_ok)) break;
      if (acc == rattle_max) { if (c == 0) atomicOr(&d.ctr->status, DEV_ERR_RATTLE); break; }
      const double den = group4_sum(gmask, dd * dP);
      double r = (double)__frcp_rn((float)den);
      r = r * (2.0 - den * r);
      r = r * (2.0 - den * r);
      const double G = -(0.25 * Con1diff * IIM) * r;
      const double hH = -(2.0 * IIM * D);
      const double u1 = G * dP + hH, u2 = hH - G * dP;
      X1 = pr1 + Q1 * dt + u1 * iMc;
      X2 = pr2 + Q2 * dt + u2 * iMn;
      if (comp) {   // every axis wraps inside the iteration (2d_array/evolve_mod.f95:365-369)
        if (X1 >= L) X1 -= L; else if (X1 < 0.0) X1 += L;
        if (X2 >= L) X2 -= L; else if (X2 < 0.0) X2 += L;
      }
      Q1 = Q1 + u1 * iMcdt;
      Q2 = Q2 + u2 * iMndt;
      acc++;
    }
    iters += acc;
    if (live && comp) {
      d.dpos[3 * s1 + c] = X1; d.dpos[3 * s2 + c] = X2;
      d.dq[3 * s1 + c] = Q1; d.dq[3 * s2 + c] = Q2;
      const double f1 = floor(X1), f2 = floor(X2);
      SphereRel<T>& r1 = d.srel[s1];
      SphereRel<T>& r2 = d.srel[s2];
      if (c == 0) { r1.cx = (int)f1; r1.ox = (T)(X1 - f1); r2.cx = (int)f2; r2.ox = (T)(X2 - f2); }
      else if (c == 1) { r1.cy = (int)f1; r1.oy = (T)(X1 - f1); r2.cy = (int)f2; r2.oy = (T)(X2 - f2); }
      else { r1.cz = (int)f1; r1.oz = (T)(X1 - f1); r2.cz = (int)f2; r2.oz = (T)(X2 - f2); }
    }
  }
  if (live && c == 0 && iters) atomicAdd(&d.ctr->rattle_iters, iters);
}

template <typename T>
void Launch<T>::dimer(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, int mode, double w3,
                      int rattle_max, cudaStream_t st) {
  if (kp.nd == 0) return;
  if (kp.rotor && sizeof(T) == 4) {
    const int threads = 4 * kp.nd;
    k_rotor_split<T><<<(threads + 31) / 32, 32, 0, st>>>(d, kp, a, mode, rattle_max);
  } else if (kp.rotor) {
    k_rotor<T><<<(kp.nd + 63) / 64, 64, 0, st>>>(d, kp, a, mode, rattle_max);
  } else if (sizeof(T) == 4) {
    // four lanes per dimer, one 32-lane block per eight dimers (spread over the SMs)
    const int threads = 4 * kp.nd;
    k_dimer_split<T><<<(threads + 31) / 32, 32, 0, st>>>(d, kp, a, mode, w3, rattle_max);
  } else {
    k_dimer<T><<<(kp.nd + 63) / 64, 64, 0, st>>>(d, kp, a, mode, w3, rattle_max);
  }
  LAUNCH_COUNT();
}

// Affected_Cell.f90:22-98 for every sphere: mark the cells near a sphere so
// the bulk reaction skips them.
template <typename T>
__global__ void k_affected(Dev<T> d, KParams<T> kp, double cutC, double cutN) {
  if (d.ctr->abort_step) return;
  const int s = blockIdx.x;
  if (s >= kp.ns) return;
  const double co = (s & 1) ? cutN : cutC, co2 = co * co;
  const double X = d.dpos[3 * s], Y = d.dpos[3 * s + 1], Z = d.dpos[3 * s + 2];
  const int lo0 = (int)ceil(X - (co + 1.0)), up0 = (int)floor(X + (co + 1.0));
  const int lo1 = (int)ceil(Y - (co + 1.0)), up1 = (int)floor(Y + (co + 1.0));
  const int lo2 = (int)ceil(Z - (co + 1.0)), up2 = (int)floor(Z + (co + 1.0));
  const int n0 = up0 - lo0 + 1, n1 = up1 - lo1 + 1, n2 = up2 - lo2 + 1;
  const int tot = n0 * n1 * n2;
  for (int q = threadIdx.x; q < tot; q += blockDim.x) {
    int i = lo0 + q % n0, j = lo1 + (q / n0) % n1, kk = lo2 + q / (n0 * n1);
    double a0 = fabs((double)(float)i - X) - 1.0;
    double b0 = fabs((double)(float)j - Y) - 1.0;
    double c0 = fabs((double)(float)kk - Z) - 1.0;
    if (a0 * a0 + b0 * b0 + c0 * c0 < co2) {
      int ci = i, cj = j, ck = kk;
      if (ci < 0) ci += kp.lx; else if (ci >= kp.lx) ci -= kp.lx;
      if (cj < 0) cj += kp.ly; else if (cj >= kp.ly) cj -= kp.ly;
      if (ck < 0) ck += kp.lz; else if (ck >= kp.lz) ck -= kp.lz;
      if (ci < 0 || ci >= kp.lx || cj < 0 || cj >= kp.ly || ck < 0 || ck >= kp.lz) continue;
      d.affected[ci + (size_t)kp.lx * (cj + (size_t)kp.ly * ck)] = 1;
    }
  }
}

template <typename T>
void Launch<T>::affected(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st) {
  if (kp.ns == 0) return;
  (void)a;
  double cutC = sqrt((double)kp.cut2[0]), cutN = sqrt((double)kp.cut2[1]);
  k_affected<T><<<kp.ns, 256, 0, st>>>(d, kp, cutC, cutN);
  LAUNCH_COUNT();
}

// Collision / distribute accumulation over the main home (used by the
// stand-alone mpc_rotation and distribute entry points).  what bit 0:
// collision, bit 1: distribute.
template <typename T>
__global__ void __launch_bounds__(TPB) k_accumulate_main(Dev<T> d, KParams<T> kp, StepArgs a, int what) {
  const T sx = step_shift<T>(a, 0), sy = step_shift<T>(a, 1), sz = step_shift<T>(a, 2);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) {
    uint32_t cell = d.p.cell[i];
    T ox = d.p.ox[i], oy = d.p.oy[i], oz = d.p.oz[i];
    uint8_t f = d.p.flag[i];
    if (what & 1) {
      uint32_t key = shifted_key(kp, cell, ox, oy, oz, sx, sy, sz);
      d.skey[i] = key;
      accum_coll<T>(d.acc, key, d.p.vx[i], d.p.vy[i], d.p.vz[i]);
    }
    if (what & 2) {
      bool inl = (f & FLAG_INLIST) != 0;
      bool bulk = true;
      if (kp.exclusion == 0 && inl) {
        int bin = bin_of(kp.lx, kp.ly, kp.nbx, kp.nby, cell);
        unsigned int nc = d.bin_cnt[bin];
        const uint16_t* bl = d.bin_list + (size_t)bin * BIN_SLOTS;
        for (unsigned int q = 0; q < nc; ++q) {
          int s = bl[q];
          T dx, dy, dz;
          if (sep2(kp, cell, ox, oy, oz, d.srel[s], dx, dy, dz) <= kp.cut2[s & 1]) bulk = false;
        }
      }
      if (bulk)
        accum_dist(d, kp, unshifted_id(kp.lx, kp.ly, cell), f & FLAG_SPECIES,
                   dist_key(kp.exclusion == 0 && inl ? 1 : 0, lid_of(d, (uint32_t)i)));
    }
  }
}

template <typename T>
void Launch<T>::accumulate_main(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, int what, cudaStream_t st) {
  k_accumulate_main<T><<<a.grid, TPB, 0, st>>>(d, kp, a, what);
  LAUNCH_COUNT();
}

// ------------------------------------------------------------ per cell ----
// Relabel the list member `key` to species `code`: in the shell buffer when
// its state lives there (the main cell[] then holds the shell slot), else in
// the main arrays.
template <typename T>
__device__ __forceinline__ void relabel_key(const Dev<T>& d, uint32_t key, int code) {
  const uint32_t idx = d.lpos ? d.lpos[key & 0x7FFFFFFFu] : key & 0x7FFFFFFFu;
  const uint8_t f = d.p.flag[idx];
  // B -> A clears the owner tag (linear_periodic_no_ci/reaction_simple_mod.f95:55)
  if (d.owner && code == 0) d.owner[idx] = 0;
  if (f & FLAG_HOME_SHELL) {
    const uint32_t j = d.p.cell[idx];
    if (!chk((int64_t)j < d.sh.cap, d.ctr, 120, j)) return;
    d.sh.flag[j] = (uint8_t)((d.sh.flag[j] & ~FLAG_SPECIES) | code);
  } else {
    d.p.flag[idx] = (uint8_t)((f & ~FLAG_SPECIES) | code);
  }
}

// Selkov six-channel RKMPC decision for one cell (RMPC_SelkovDimer.f90:132-321)
// in FP64: channel 1..6 or 0.
static __device__ int selkov_channel_fp64(const double* k, double tau, int nF, int nG, int nI, double x1, double x2) {
  double a1 = k[0], a2 = k[1] * (double)nF, a5 = k[4] * (double)nG, a6 = k[5];
  double a3 = (nG == 0) ? 0. : k[2] * (double)nF * (double)nG * (double)(nG - 1);
  double a4 = (nG <= 1) ? 0. : k[3] * (double)nG * (double)(nG - 1) * (double)(nG - 2);
  if (nI == 0) { a1 = 0.; a6 = 0.; }
  double a00 = a1 + a2 + a3 + a4 + a5 + a6;
  double prob = 1 - exp(-a00 * tau);
  if (!(prob > x2)) return 0;
  if (nI == 0 && nF == 0 && nG == 0) return 0;
  double a0rand = a00 * x1;
  double av[6] = {a1, a2, a3, a4, a5, a6};
  double cum = 0.;
  for (int c = 0; c < 6; ++c) {
    cum = cum + av[c];
    if (av[c] != 0. && a0rand < cum) return c + 1;
  }
  return 0;
}

// The same decision in FP32 with a guard band; returns -1 when any comparison
// is too close to call in FP32 (the caller then uses the FP64 path).  The
// uniforms come in as floats of the leading 32 bits of the draws (within
// 1e-7 of the 53-bit values, far inside the band).
static __device__ int selkov_channel_fp32(const float* kf, float tau, int nF, int nG, int nI, float x1, float x2) {
  const float k0 = kf[0], k1 = kf[1], k2 = kf[2], k3 = kf[3], k4 = kf[4], k5 = kf[5];
  float a1 = k0, a2 = k1 * (float)nF, a5 = k4 * (float)nG, a6 = k5;
  float a3 = (nG == 0) ? 0.f : k2 * (float)nF * (float)nG * (float)(nG - 1);
  float a4 = (nG <= 1) ? 0.f : k3 * (float)nG * (float)(nG - 1) * (float)(nG - 2);
  if (nI == 0) { a1 = 0.f; a6 = 0.f; }
  float a00 = a1 + a2 + a3 + a4 + a5 + a6;
  float prob = 1.f - expf(-a00 * tau);
  float gap = prob - x2;
  if (fabsf(gap) < 4e-6f) return -1;
  if (!(gap > 0.f)) return 0;
  if (nI == 0 && nF == 0 && nG == 0) return 0;
  float a0rand = a00 * x1;
  float av[6] = {a1, a2, a3, a4, a5, a6};
  float cum = 0.f;
  const float band = 4e-6f * a00 + 1e-30f;
  for (int c = 0; c < 6; ++c) {
    cum = cum + av[c];
    if (av[c] != 0.f) {
      if (fabsf(a0rand - cum) < band) return -1;
      if (a0rand < cum) return c + 1;
    }
  }
  return 0;
}

// One thread per cell after a collision step: centre-of-mass velocity and
// random axis of every shifted cell (mpc_rotation_mod.f95:163-194), the bulk
// reaction of every unshifted cell (reaction_mod.f95:41-62 or
// RMPC_SelkovDimer.f90:127-324) and the reset of the accumulators.
// what bit 0: collision tables, bit 1: reaction.
template <typename T>
__global__ void __launch_bounds__(TPB, 6) k_cells(Dev<T> d, KParams<T> kp, StepArgs a, int what) {
  if (d.ctr->abort_step) return;
  const int64_t nmax = kp.ncell_shift > kp.ncell ? kp.ncell_shift : kp.ncell;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const double pi = 3.141592653589793;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nmax; c += stride) {
    if ((what & 1) && c < kp.ncell_shift) {
      T cmx = (T)0, cmy = (T)0, cmz = (T)0;
      if (sizeof(T) == 4) {
        float4* ac = reinterpret_cast<float4*>(d.acc) + c;
        float4 v = *ac;
        if (v.x != 0.f) {
          if (kp.rotation_sense > 0) { cmx = (T)(v.y / v.x); cmy = (T)(v.z / v.x); cmz = (T)(v.w / v.x); }
          else { float inv = 1.f / v.x; cmx = (T)(v.y * inv); cmy = (T)(v.z * inv); cmz = (T)(v.w * inv); }
        }
        *ac = make_float4(0.f, 0.f, 0.f, 0.f);
      } else {
        double* ac = reinterpret_cast<double*>(d.acc) + 4 * (size_t)c;
        double n = ac[0];
        if (n != 0.) {
          if (kp.rotation_sense > 0) { cmx = (T)(ac[1] / n); cmy = (T)(ac[2] / n); cmz = (T)(ac[3] / n); }
          else { double inv = 1.0 / n; cmx = (T)(ac[1] * inv); cmy = (T)(ac[2] * inv); cmz = (T)(ac[3] * inv); }
        }
        ac[0] = ac[1] = ac[2] = ac[3] = 0.;
      }
      T ux, uy, uz;
      if (sizeof(T) == 4) {
        // FP32 axis from the top 32 bits of each draw; the radius is
        // 2 sqrt(u (1 - u)) = sqrt(1 - theta^2) with both factors at full
        // relative precision (no cancellation near the poles)
        uint32_t w0, w2;
        contract_words(kp.seed, TAG_AXIS, (uint32_t)c, 0, a.step, w0, w2);
        const float two32 = 2.3283064365386963e-10f;
        float u1 = (float)w0 * two32;
        float u2 = (float)w2 * two32, v2 = ((float)(~w2) + 1.f) * two32;
        float sp, cp;
        sincospif(2.f * u1, &sp, &cp);
        float th = u2 - v2;
        float r = 2.f * sqrtf(u2 * v2);
        ux = (T)(r * cp); uy = (T)(r * sp); uz = (T)th;
      } else {
        double u1, u2;
        contract_pair(kp.seed, TAG_AXIS, (uint32_t)c, 0, a.step, u1, u2);
        double phi = 2.0 * pi * u1, theta = 2.0 * u2 - 1.0;
        ux = (T)(sqrt(1.0 - theta * theta) * cos(phi));
        uy = (T)(sqrt(1.0 - theta * theta) * sin(phi));
        uz = (T)theta;
      }
      T* r = d.rot + 6 * (size_t)c;
      r[0] = cmx; r[1] = cmy; r[2] = cmz; r[3] = ux; r[4] = uy; r[5] = uz;
    }
    if ((what & 2) && c < kp.ncell) {
      unsigned int cnt = d.dcnt[c];
      uint32_t* fk = d.dfirst + 4 * (size_t)c;
      if (kp.kinetics == 1) {
        int nB = (cnt >> 8) & 255u;
        if (nB > 0) {
          bool fire;
          bool exact = sizeof(T) != 4;
          if (!exact) {
            // FP32 with a guard band on the leading word of the draw; a call
            // too close to make (or a zero word) takes the FP64 path
            uint32_t w0, w2;
            contract_words(kp.seed, TAG_RXN, (uint32_t)c, 0, a.step, w0, w2);
            const float u0f = (float)w0 * 2.3283064365386963e-10f;
            const float pf = 1.f - expf(-(kp.kf[0] * (float)nB) * kp.tauf);
            const float g = pf - u0f;
            exact = fabsf(g) < 4e-6f || w0 == 0u;
            fire = g >= 0.f;
          }
          if (exact) {
            double u0, u1;
            contract_pair(kp.seed, TAG_RXN, (uint32_t)c, 0, a.step, u0, u1);
            const double a1 = kp.k[0] * (double)nB;
            fire = (0. < u0 && u0 <= 1.0 - exp(-a1 * kp.tau));
          }
          if (fire && fk[1] != 0xFFFFFFFFu) relabel_key(d, fk[1], 0);
        }
      } else if (kp.kinetics == 2 && !d.affected[c]) {
        // channel 1..6 -> species relabelled (target) and its new code, one
        // nibble per channel (RMPC_SelkovDimer.f90:132-321): targets 3 0 0 1 1 3,
        // codes 0 3 1 0 3 1 (register constants instead of a local table)
        const unsigned tgt_nib = 0x3110030u, code_nib = 0x1301300u;
        int nF = cnt & 255u, nG = (cnt >> 8) & 255u, nI = (cnt >> 24) & 255u;
        int ch = -1;
        if (sizeof(T) == 4) {
          uint32_t w1, w2;
          contract_words(kp.seed, TAG_RXN, (uint32_t)c, 0, a.step, w1, w2);
          const float two32 = 2.3283064365386963e-10f;
          ch = selkov_channel_fp32(kp.kf, kp.tauf, nF, nG, nI, (float)w1 * two32, (float)w2 * two32);
        }
        if (ch < 0) {
          double x1, x2;
          contract_pair(kp.seed, TAG_RXN, (uint32_t)c, 0, a.step, x1, x2);
          ch = selkov_channel_fp64(kp.k, kp.tau, nF, nG, nI, x1, x2);
        }
        if (ch > 0) {
          const uint32_t key = fk[(tgt_nib >> (4 * ch)) & 0xFu];
          if (key != 0xFFFFFFFFu) relabel_key(d, key, (int)((code_nib >> (4 * ch)) & 0xFu));
        }
      }
      d.dcnt[c] = 0u;
      *reinterpret_cast<uint4*>(fk) = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
      d.affected[c] = 0;
    }
  }
}

template <typename T>
void Launch<T>::cells(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, int what, cudaStream_t st) {
  k_cells<T><<<a.g_cells > 0 ? a.g_cells : a.grid, TPB, 0, st>>>(d, kp, a, what);
  LAUNCH_COUNT();
}

// Watch list support: for every coarse bin, a lower bound on the distance
// from any point of the bin to the list radius (r_c 2^(1/6) + skin) of any
// sphere, clamped at 0 (float bits, so atomicMin orders them).  Bins farther
// than the largest flight of the coming period keep the initial huge value.
template <typename T>
__global__ void k_gap_fill(Dev<T> d, KParams<T> kp, double Rc, double Rn, int horizon) {
  const int s = blockIdx.x;
  if (s >= kp.ns) return;
  const double Rl = (s & 1) ? Rn : Rc;
  // |v'| <= |v| + 2 |v_cm| <= 3 vmax after the collision (vmax of the last
  // rebuild); the spheres move at most vs; one cell of margin
  const double vmax = sqrt(__longlong_as_double((long long)d.ctr->vlast));
  const double vs = (double)sphere_speed_bound<T>(d.ctr);
  const double reach = (3.0 * vmax + vs) * kp.dtd * (double)horizon + 1.0;
  const double hd = 0.5 * sqrt(3.0) * (double)GAP_EDGE;
  const double Rm = Rl + reach + hd;
  const int nb[3] = {kp.ngx, kp.ngy, kp.ngz};
  const double L[3] = {(double)kp.lx, (double)kp.ly, (double)kp.lz};
  const bool per[3] = {true, true, kp.geometry == 1};
  double X[3];
  int lo[3], hi[3];
  for (int q = 0; q < 3; ++q) {
    X[q] = d.dpos[3 * s + q];
    lo[q] = (int)floor((X[q] - Rm) / (double)GAP_EDGE);
    hi[q] = (int)floor((X[q] + Rm) / (double)GAP_EDGE);
    if (!per[q]) { lo[q] = max(lo[q], 0); hi[q] = min(hi[q], nb[q] - 1); }
    else if (hi[q] - lo[q] + 1 >= nb[q]) { lo[q] = 0; hi[q] = nb[q] - 1; }
  }
  const int n0 = hi[0] - lo[0] + 1, n1 = hi[1] - lo[1] + 1, n2 = hi[2] - lo[2] + 1;
  const int tot = n0 * n1 * n2;
  // the per-bin arithmetic in FP32 (FP64 is slow on this part), with a
  // margin of 1e-3 cells that keeps the bound below the exact one
  const float Xf[3] = {(float)X[0], (float)X[1], (float)X[2]};
  const float Lf[3] = {(float)L[0], (float)L[1], (float)L[2]};
  const float sub = (float)(hd + Rl) + 1e-3f;
  for (int t = threadIdx.x; t < tot; t += blockDim.x) {
    int w[3] = {lo[0] + t % n0, lo[1] + (t / n0) % n1, lo[2] + t / (n0 * n1)};
    float d2 = 0.f;
    for (int q = 0; q < 3; ++q) {
      if (per[q]) { if (w[q] < 0) w[q] += nb[q]; else if (w[q] >= nb[q]) w[q] -= nb[q]; }
      float dc = (float)(w[q] * GAP_EDGE) + 0.5f * (float)GAP_EDGE - Xf[q];
      if (per[q]) dc = min_image(dc, Lf[q]);
      d2 += dc * dc;
    }
    float lb = sqrtf(d2) - sub;
    if (lb < 0.f) lb = 0.f;
    const int b = w[0] + nb[0] * (w[1] + nb[1] * w[2]);
    if (!chk(b >= 0 && b < nb[0] * nb[1] * nb[2], d.ctr, 122, b)) continue;
    atomicMin(&d.gapf[b], __float_as_uint(lb));
  }
}

template <typename T>
void Launch<T>::gap_field(const Dev<T>& d, const KParams<T>& kp, int horizon, cudaStream_t st) {
  const int nbins = kp.ngx * kp.ngy * kp.ngz;
  cudaMemsetAsync(d.gapf, 0x7F, sizeof(uint32_t) * nbins, st);   // 3.4e38
  if (kp.ns == 0) return;
  const double Rc = sqrt((double)kp.full2[0]) + 1e-6, Rn = sqrt((double)kp.full2[1]) + 1e-6;
  k_gap_fill<T><<<kp.ns, 256, 0, st>>>(d, kp, Rc, Rn, horizon);
  LAUNCH_COUNT();
}

// Watch-list test of an outside particle after the collision: can it come
// within the list radius of a sphere (gap: the gap field of its bin), or hit
// a wall, before the next collision (`horizon` steps at speed sqrt(v2))?
template <typename T>
__device__ __forceinline__ bool watch_test(const KParams<T>& kp, T gap, uint32_t cell, T vz, T v2, int horizon,
                                           T vs) {
  const T t = kp.dt * (T)horizon;
  if (gap < (T)1e30 && gap <= (sqrt(v2) + vs) * t + (T)0.1) return true;
  if (kp.geometry == 0) {
    const T cz = (T)cell_z(cell), dz = fabs(vz) * t;
    if (cz - dz < (T)0.05 || cz + (T)1 + dz > (T)kp.lz - (T)0.05) return true;
  }
  return false;
}

template <typename T>
__global__ void __launch_bounds__(TPB) k_rotate_main(Dev<T> d, KParams<T> kp, StepArgs a) {
  if (d.ctr->abort_step) return;
  // two particles per thread and iteration: all loads and both table gathers
  // are issued before the first store
  T vmax2 = (T)0;   // speed bound of the outside particles until the next collision
  // with a.watch_build (= the period in steps): the particles that can come
  // near a sphere or a wall before the next collision join the watch list;
  // vfar2 is the largest v^2 of the others (constant until that collision)
  T vfar2 = (T)0;
  const T vs = sphere_speed_bound<T>(d.ctr);
  // watch-list appends staged per warp (the loop is warp-uniform)
  __shared__ uint32_t wl_buf[(TPB / 32) * WL_CAP];
  uint32_t* wbuf = wl_buf + (threadIdx.x >> 5) * WL_CAP;
  unsigned wn = 0;
  const int lane = threadIdx.x & 31;
  // blocks take tiles of ROT_TILE consecutive particles in a grid stride (two
  // 256-particle steps per iteration), so that the watch list a warp stages
  // keeps the particles' cell order
  // (32-bit indices: particle counts are below 2^31)
  constexpr int ROT_STEPS = 16;
  constexpr uint32_t ROT_TILE = (uint32_t)ROT_STEPS * TPB;
  const uint32_t n32 = (uint32_t)kp.n;
  const uint32_t tile_stride = gridDim.x * ROT_TILE;
  int step = 0;
  for (uint32_t i0 = blockIdx.x * ROT_TILE + threadIdx.x; i0 - lane < n32;
       i0 = step + 2 < ROT_STEPS ? i0 + 2 * TPB : i0 - (uint32_t)(ROT_STEPS - 2) * TPB + tile_stride,
       step = step + 2 < ROT_STEPS ? step + 2 : 0) {
    const uint32_t i1 = i0 + TPB;
    const bool h0 = i0 < n32;
    const bool h1 = i1 < n32;
    bool w0 = false, w1 = false;
    const uint8_t f0 = h0 ? d.p.flag[i0] : FLAG_HOME_SHELL;
    const uint8_t f1 = h1 ? d.p.flag[i1] : FLAG_HOME_SHELL;
    const uint32_t k0 = h0 ? d.skey[i0] : 0u;
    const uint32_t k1 = h1 ? d.skey[i1] : 0u;
    T vx0 = (T)0, vy0 = (T)0, vz0 = (T)0;
    if (h0) { vx0 = d.p.vx[i0]; vy0 = d.p.vy[i0]; vz0 = d.p.vz[i0]; }
    T vx1 = (T)0, vy1 = (T)0, vz1 = (T)0;
    if (h1) { vx1 = d.p.vx[i1]; vy1 = d.p.vy[i1]; vz1 = d.p.vz[i1]; }
    const bool r0 = !(f0 & FLAG_HOME_SHELL), r1 = !(f1 & FLAG_HOME_SHELL);
    // watch-list inputs, loaded with the rest before any store
    uint32_t c0 = 0, c1 = 0;
    if (a.watch_build) {
      if (r0) c0 = d.p.cell[i0];
      if (r1) c1 = d.p.cell[i1];
    }
    T t0[6] = {}, t1[6] = {};
    if (r0) load_rot(d.rot, k0, t0);
    if (r1) load_rot(d.rot, k1, t1);
    T g0 = (T)3e38, g1 = (T)3e38;
    if (a.watch_build) {
      if (r0) g0 = __uint_as_float(d.gapf[gap_bin_of(kp.ngx, kp.ngy, c0)]);
      if (r1) g1 = __uint_as_float(d.gapf[gap_bin_of(kp.ngx, kp.ngy, c1)]);
    }
    if (r0) {
      rotate_v(kp, t0, vx0, vy0, vz0);
      d.p.vx[i0] = vx0; d.p.vy[i0] = vy0; d.p.vz[i0] = vz0;
      const T w = vx0 * vx0 + vy0 * vy0 + vz0 * vz0;
      vmax2 = w > vmax2 ? w : vmax2;
      if (a.watch_build) {
        w0 = watch_test(kp, g0, c0, vz0, w, a.watch_build, vs);
        if (!w0) vfar2 = w > vfar2 ? w : vfar2;
      }
    }
    if (r1) {
      rotate_v(kp, t1, vx1, vy1, vz1);
      d.p.vx[i1] = vx1; d.p.vy[i1] = vy1; d.p.vz[i1] = vz1;
      const T w = vx1 * vx1 + vy1 * vy1 + vz1 * vz1;
      vmax2 = w > vmax2 ? w : vmax2;
      if (a.watch_build) {
        w1 = watch_test(kp, g1, c1, vz1, w, a.watch_build, vs);
        if (!w1) vfar2 = w > vfar2 ? w : vfar2;
      }
    }
    if (a.watch_build) {
      wl_add(wbuf, wn, w0, (uint32_t)i0, &d.ctr->n_watch, d.watch);
      wl_add(wbuf, wn, w1, (uint32_t)i1, &d.ctr->n_watch, d.watch);
    }
  }
  if (a.watch_build) wl_flush(wbuf, wn, &d.ctr->n_watch, d.watch);
  block_max_to<T>(&d.ctr->vpost, vmax2);
  if (a.watch_build) {
    __syncthreads();   // block_max_to's shared buffer is reused
    block_max_to<T>(&d.ctr->vfar, vfar2);
  }
}

template <typename T>
void Launch<T>::rotate_main(const Dev<T>& d, const KParams<T>& kp, const StepArgs& a, cudaStream_t st) {
  k_rotate_main<T><<<a.g_rotate, TPB, 0, st>>>(d, kp, a);
  LAUNCH_COUNT();
}

template <typename T>
void Launch<T>::occupancy(int* blocks) {
  blocks[0] = blocks[1] = blocks[2] = blocks[3] = blocks[4] = blocks[5] = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[0], k_rebuild<T>, TPB, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[1], k_force<T, false>, TPB, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[2], k_rotate_main<T>, TPB, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[3], k_rebuild_far<T>, TPB, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[4], k_cells<T>, TPB, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks[5], k_shell_advance<T>, TPB, 0);
}

// ---------------------------------------------------- shell home moves ----
template <typename T>
__global__ void k_flush(Dev<T> d, KParams<T> kp) {
  const unsigned int nin = d.ctr->n_inside;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < (int64_t)nin; j += stride) {
    uint32_t i = d.sh.idx[j];
    d.p.cell[i] = d.sh.cell[j];
    d.p.ox[i] = d.sh.ox[j]; d.p.oy[i] = d.sh.oy[j]; d.p.oz[i] = d.sh.oz[j];
    d.p.vx[i] = d.sh.vx[j]; d.p.vy[i] = d.sh.vy[j]; d.p.vz[i] = d.sh.vz[j];
    d.p.flag[i] = (d.sh.flag[j] & FLAG_SPECIES) | FLAG_INLIST;
  }
}

template <typename T>
void Launch<T>::flush(const Dev<T>& d, const KParams<T>& kp, cudaStream_t st) {
  k_flush<T><<<512, TPB, 0, st>>>(d, kp);
  LAUNCH_COUNT();
}

template <typename T>
__global__ void k_regather(Dev<T> d, KParams<T> kp) {
  const unsigned int nin = d.ctr->n_inside;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < (int64_t)nin; j += stride) {
    uint32_t i = d.sh.idx[j];
    d.sh.cell[j] = d.p.cell[i];
    d.sh.ox[j] = d.p.ox[i]; d.sh.oy[j] = d.p.oy[i]; d.sh.oz[j] = d.p.oz[i];
    d.sh.vx[j] = d.p.vx[i]; d.sh.vy[j] = d.p.vy[i]; d.sh.vz[j] = d.p.vz[i];
    d.sh.flag[j] = (d.p.flag[i] & FLAG_SPECIES) | FLAG_INLIST;
    d.p.cell[i] = (uint32_t)j;
    d.p.flag[i] = (d.p.flag[i] & FLAG_SPECIES) | FLAG_INLIST | FLAG_HOME_SHELL;
  }
}

template <typename T>
void Launch<T>::regather(const Dev<T>& d, const KParams<T>& kp, cudaStream_t st) {
  k_regather<T><<<512, TPB, 0, st>>>(d, kp);
  LAUNCH_COUNT();
}

// ------------------------------------------------------------------ sort ----
// sort_hilbert_mod.f95:6-98: stable counting sort of all particles by the
// visiting rank of their cell (bucket fill, per-cell index sort, gather).
template <typename T>
__global__ void k_sort_count(Dev<T> d, KParams<T> kp) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) {
    uint32_t cid = unshifted_id(kp.lx, kp.ly, d.p.cell[i]);
    if (!chk(cid < (uint32_t)kp.ncell, d.ctr, 101, cid)) continue;
    uint32_t r = d.order_rank[cid];
    if (!chk(r < (uint32_t)kp.ncell, d.ctr, 102, r)) continue;
    atomicAdd(&d.scnt[r], 1u);
  }
}

template <typename T>
__global__ void k_sort_fill(Dev<T> d, KParams<T> kp) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) {
    uint32_t cid = unshifted_id(kp.lx, kp.ly, d.p.cell[i]);
    if (!chk(cid < (uint32_t)kp.ncell, d.ctr, 103, cid)) continue;
    uint32_t r = d.order_rank[cid];
    if (!chk(r < (uint32_t)kp.ncell, d.ctr, 104, r)) continue;
    uint32_t pos = d.sstart[r] + atomicAdd(&d.sfill[r], 1u);
    if (!chk(pos < (uint32_t)kp.n, d.ctr, 105, pos)) continue;
    d.sidx[pos] = (uint32_t)i;
  }
}

template <typename T>
__global__ void k_sort_segments(Dev<T> d, KParams<T> kp) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < kp.ncell; r += stride) {
    uint32_t b = d.sstart[r], n = d.scnt[r];
    if (!chk((int64_t)b + n <= kp.n, d.ctr, 106, (long long)b + n)) continue;
    // by main index: the slots of re-sorted particles are not in index order
    uint32_t* s = d.sidx + b;
    for (uint32_t i = 1; i < n; ++i) {
      const uint32_t v = s[i], kv = lid_of(d, v);
      int j = (int)i - 1;
      while (j >= 0 && lid_of(d, s[j]) > kv) { s[j + 1] = s[j]; --j; }
      s[j + 1] = v;
    }
  }
}

template <typename T>
__global__ void k_sort_gather(Dev<T> d, KParams<T> kp) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < kp.n; q += stride) {
    uint32_t i = d.sidx[q];
    if (!chk(i < (uint32_t)kp.n, d.ctr, 107, i)) continue;
    d.p2.cell[q] = d.p.cell[i];
    d.p2.ox[q] = d.p.ox[i]; d.p2.oy[q] = d.p.oy[i]; d.p2.oz[q] = d.p.oz[i];
    d.p2.vx[q] = d.p.vx[i]; d.p2.vy[q] = d.p.vy[i]; d.p2.vz[q] = d.p.vz[i];
    d.p2.flag[q] = d.p.flag[i] & FLAG_SPECIES;
    if (d.owner) d.owner2[q] = d.owner[i];
    if (d.inc) d.inc2[q] = d.inc[i];
  }
}

// Order-only re-sort.  The reference keeps its arrays in index order between
// sorts; here particles may move to other slots in between, keeping their
// main index (lid / lpos), so that the slots follow the cell order while the
// particles diffuse.  It runs at the start of a collision step's rebuild and
// groups every particle by the sort rank of the cell it is in at that step
// (a shell-resident particle: its shell cell; a lazily streamed one: its
// stored state streamed over its lag, the same flight the collision pass
// then makes), in any order inside a cell.  The records move as stored
// (lagging states and flags included), and a shell slot learns its
// member's new slot.
//
// Two levels, so that no pass needs an atomic per particle: bins of 2^bits
// consecutive ranks (up to a thousand particles on average; a warp of the
// nearly sorted slots meets one or two bins, one aggregated atomic each),
// then a counting sort of each bin in shared memory.  Scratch: the rank of
// every slot in skey, the bin lists (slot, rank) in sidx / watch; none of
// them is live at the start of a collision step's rebuild.
constexpr int RESORT_MAX_BITS = 8;   // at most 256 ranks per bin (one per thread of the fine pass)
constexpr int RESORT_UNROLL = 4;     // 32-particle steps per warp with their loads issued first
constexpr int RESORT_CAP = 2048;     // members of a bin sorted in shared memory (larger: bin order kept)

template <typename T>
__global__ void k_resort_count(Dev<T> d, KParams<T> kp, int bits, int tc, int tc_full) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x * RESORT_UNROLL;
  for (int64_t base = (blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31)) * RESORT_UNROLL; base < kp.n;
       base += stride) {
    uint32_t c[RESORT_UNROLL];
    uint8_t f[RESORT_UNROLL];
    T ox[RESORT_UNROLL], oy[RESORT_UNROLL], oz[RESORT_UNROLL], vx[RESORT_UNROLL], vy[RESORT_UNROLL], vz[RESORT_UNROLL];
#pragma unroll
    for (int u = 0; u < RESORT_UNROLL; ++u) {
      const int64_t i = base + 32 * u + lane;
      c[u] = 0u; f[u] = FLAG_INLIST;
      ox[u] = oy[u] = oz[u] = vx[u] = vy[u] = vz[u] = (T)0;
      if (i < kp.n) {
        c[u] = d.p.cell[i]; f[u] = d.p.flag[i];
        ox[u] = d.p.ox[i]; oy[u] = d.p.oy[i]; oz[u] = d.p.oz[i];
        vx[u] = d.p.vx[i]; vy[u] = d.p.vy[i]; vz[u] = d.p.vz[i];
      }
    }
    uint32_t r[RESORT_UNROLL];
#pragma unroll
    for (int u = 0; u < RESORT_UNROLL; ++u) {
      if (f[u] & FLAG_HOME_SHELL) {
        if (!chk((int64_t)c[u] < d.sh.cap, d.ctr, 130, c[u])) c[u] = 0;
        c[u] = d.sh.cell[c[u]];
      } else if (!(f[u] & FLAG_INLIST)) {
        // the lag of k_rebuild / k_rebuild_far
        const int lag = (f[u] & (FLAG_FRESH | FLAG_PASSIVE)) ? tc : tc_full;
        if (lag > 0) {
          uint8_t ff = f[u] & FLAG_SPECIES;
          stream_one(kp, d.react_box, c[u], ox[u], oy[u], oz[u], vx[u], vy[u], vz[u], ff, true, lag);
        }
      }
      uint32_t cid = unshifted_id(kp.lx, kp.ly, c[u]);
      if (!chk(cid < (uint32_t)kp.ncell, d.ctr, 131, cid)) cid = 0;
      r[u] = base + 32 * u + lane < kp.n ? d.order_rank[cid] : 0u;
    }
#pragma unroll
    for (int u = 0; u < RESORT_UNROLL; ++u) {
      const int64_t i = base + 32 * u + lane;
      const bool act = i < kp.n;
      const unsigned am = __ballot_sync(0xffffffffu, act);
      if (!act) continue;
      d.skey[i] = r[u];
      const uint32_t b = r[u] >> bits;
      const unsigned peers = __match_any_sync(am, b);
      if (lane == __ffs(peers) - 1) atomicAdd(&d.scnt[b], (unsigned)__popc(peers));
    }
  }
}

template <typename T>
__global__ void k_resort_bin(Dev<T> d, KParams<T> kp, int bits) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x * RESORT_UNROLL;
  for (int64_t base = (blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31)) * RESORT_UNROLL; base < kp.n;
       base += stride) {
    uint32_t r[RESORT_UNROLL];
#pragma unroll
    for (int u = 0; u < RESORT_UNROLL; ++u) {
      const int64_t i = base + 32 * u + lane;
      r[u] = i < kp.n ? d.skey[i] : 0u;
    }
    // the groups of all four steps first, then their atomics (independent,
    // all in flight at once), then the placements
    unsigned peers[RESORT_UNROLL], am[RESORT_UNROLL];
    uint32_t pos[RESORT_UNROLL];
#pragma unroll
    for (int u = 0; u < RESORT_UNROLL; ++u) {
      const bool act = base + 32 * u + lane < kp.n;
      am[u] = __ballot_sync(0xffffffffu, act);
      peers[u] = act ? __match_any_sync(am[u], r[u] >> bits) : 0u;
    }
#pragma unroll
    for (int u = 0; u < RESORT_UNROLL; ++u) {
      pos[u] = 0u;
      if (peers[u] && lane == __ffs(peers[u]) - 1) {
        const uint32_t b = r[u] >> bits;
        pos[u] = d.sstart[b] + atomicAdd(&d.sfill[b], (unsigned)__popc(peers[u]));
      }
    }
#pragma unroll
    for (int u = 0; u < RESORT_UNROLL; ++u) {
      if (!peers[u]) continue;   // (lanes past the end; the others are exactly am[u])
      const uint32_t p0 = __shfl_sync(am[u], pos[u], __ffs(peers[u]) - 1);
      const int64_t i = base + 32 * u + lane;
      const uint32_t q = p0 + (uint32_t)__popc(peers[u] & ((1u << lane) - 1u));
      if (!chk(q < (uint32_t)kp.n, d.ctr, 132, q)) continue;
      d.sidx[q] = (uint32_t)i;
      d.watch[q] = r[u];
    }
  }
}

// A particle's record in the main arrays (moved whole by the re-sort).
template <typename T>
struct Rec {
  uint32_t cell, id;
  T ox, oy, oz, vx, vy, vz;
  uint8_t flag, inc;
  uint16_t owner;
};

template <typename T>
__device__ __forceinline__ Rec<T> rec_load(const Dev<T>& d, uint32_t i) {
  Rec<T> r;
  r.cell = d.p.cell[i];
  r.ox = d.p.ox[i]; r.oy = d.p.oy[i]; r.oz = d.p.oz[i];
  r.vx = d.p.vx[i]; r.vy = d.p.vy[i]; r.vz = d.p.vz[i];
  r.flag = d.p.flag[i];
  r.inc = d.inc ? d.inc[i] : 0;
  r.owner = d.owner ? d.owner[i] : 0;
  r.id = lid_of(d, i);
  return r;
}

template <typename T>
__device__ __forceinline__ void rec_store(const Dev<T>& d, const Rec<T>& r, uint32_t q) {
  d.p2.cell[q] = r.cell;
  d.p2.ox[q] = r.ox; d.p2.oy[q] = r.oy; d.p2.oz[q] = r.oz;
  d.p2.vx[q] = r.vx; d.p2.vy[q] = r.vy; d.p2.vz[q] = r.vz;
  d.p2.flag[q] = r.flag;
  if (d.inc) d.inc2[q] = r.inc;
  if (d.owner) d.owner2[q] = r.owner;
  d.lid2[q] = r.id;
  d.lpos[r.id] = q;
  if (r.flag & FLAG_HOME_SHELL) d.sh.idx[r.cell] = q;
}

// One block per bin (grid stride over the bins): the bin's (slot, rank)
// list is staged in shared memory with coalesced loads, counted and ranked
// there (a counting sort), and then the block writes the bin's new slots in
// order (whole sectors), each thread gathering its records with all loads
// in flight before the stores.
template <typename T>
__global__ void __launch_bounds__(TPB, 3) k_resort_fine(Dev<T> d, KParams<T> kp, int bits, int nbins) {
  constexpr int PER = RESORT_CAP / TPB;   // members per thread
  __shared__ uint32_t s_src[RESORT_CAP];
  __shared__ uint16_t s_key[RESORT_CAP];
  __shared__ uint32_t s_perm[RESORT_CAP];
  __shared__ uint32_t s_off[1 << RESORT_MAX_BITS];
  __shared__ uint32_t s_wsum[TPB / 32];
  const int W = 1 << bits;
  const uint32_t mask = (uint32_t)W - 1u;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b = blockIdx.x; b < nbins; b += gridDim.x) {
    const uint32_t start = d.sstart[b], n = d.scnt[b];
    if (n > (uint32_t)RESORT_CAP) {
      // (far above the mean) keep the bin order: still a valid permutation
      for (uint32_t t = threadIdx.x; t < n; t += TPB) {
        const uint32_t i = d.sidx[start + t];
        if (chk(i < (uint32_t)kp.n, d.ctr, 134, (long long)i)) rec_store(d, rec_load(d, i), start + t);
      }
      __syncthreads();
      continue;
    }
    if (threadIdx.x < W) s_off[threadIdx.x] = 0u;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const uint32_t t = threadIdx.x + k * TPB;
      if (t < n) { s_src[t] = d.sidx[start + t]; s_key[t] = (uint16_t)(d.watch[start + t] & mask); }
    }
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < n; t += TPB) atomicAdd(&s_off[s_key[t]], 1u);
    __syncthreads();
    // exclusive scan of the W <= TPB counts
    const uint32_t v = threadIdx.x < W ? s_off[threadIdx.x] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_wsum[warp] = x;
    __syncthreads();
    uint32_t before = 0u;
    for (int w = 0; w < warp; ++w) before += s_wsum[w];
    if (threadIdx.x < W) s_off[threadIdx.x] = before + x - v;
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < n; t += TPB) s_perm[atomicAdd(&s_off[s_key[t]], 1u)] = s_src[t];
    __syncthreads();
    constexpr int G = 4;   // records in flight per thread
#pragma unroll 1
    for (int k0 = 0; k0 < PER; k0 += G) {
      if (threadIdx.x + k0 * TPB >= n) break;
      Rec<T> rec[G];
#pragma unroll
      for (int k = 0; k < G; ++k) {
        const uint32_t t = threadIdx.x + (k0 + k) * TPB;
        if (t < n) {
          const uint32_t i = s_perm[t];
          if (chk(i < (uint32_t)kp.n, d.ctr, 135, (long long)i)) rec[k] = rec_load(d, i);
        }
      }
#pragma unroll
      for (int k = 0; k < G; ++k) {
        const uint32_t t = threadIdx.x + (k0 + k) * TPB;
        if (t < n) rec_store(d, rec[k], start + t);
      }
    }
    __syncthreads();
  }
}

template <typename T>
void Launch<T>::resort(Dev<T>& d, const KParams<T>& kp, int tc, int tc_full, cudaStream_t st) {
  // bins of 2^bits ranks holding at most 3/4 of the fine pass's capacity on
  // average (larger bins spread the fine pass's fixed cost per bin over more
  // particles; a bin's Poisson spread stays far below the capacity)
  const double per_cell = (double)kp.n / (double)kp.ncell;
  int bits = 0;
  while (bits < RESORT_MAX_BITS && (double)(2 << bits) * per_cell <= 0.75 * RESORT_CAP) ++bits;
  const int nbins = (int)((kp.ncell + (1 << bits) - 1) >> bits);
  cudaMemsetAsync(d.scnt, 0, sizeof(uint32_t) * nbins, st);
  cudaMemsetAsync(d.sfill, 0, sizeof(uint32_t) * nbins, st);
  k_resort_count<T><<<1024, TPB, 0, st>>>(d, kp, bits, tc, tc_full);
  scan_u32(d.scnt, d.sstart, nbins, d.scan_tmp, st);
  k_resort_bin<T><<<1024, TPB, 0, st>>>(d, kp, bits);
  k_resort_fine<T><<<nbins < 65535 ? nbins : 65535, TPB, 0, st>>>(d, kp, bits, nbins);
  LAUNCH_COUNT(); LAUNCH_COUNT(); LAUNCH_COUNT();
  Particles<T> t = d.p; d.p = d.p2; d.p2 = t;
  uint16_t* o = d.owner; d.owner = d.owner2; d.owner2 = o;
  uint8_t* c = d.inc; d.inc = d.inc2; d.inc2 = c;
  uint32_t* l = d.lid; d.lid = d.lid2; d.lid2 = l;
}

template <typename T>
void Launch<T>::sort(Dev<T>& d, const KParams<T>& kp, cudaStream_t st) {
  cudaMemsetAsync(d.scnt, 0, sizeof(uint32_t) * kp.ncell, st);
  cudaMemsetAsync(d.sfill, 0, sizeof(uint32_t) * kp.ncell, st);
  k_sort_count<T><<<1024, TPB, 0, st>>>(d, kp);
  scan_u32(d.scnt, d.sstart, kp.ncell, d.scan_tmp, st);
  k_sort_fill<T><<<1024, TPB, 0, st>>>(d, kp);
  k_sort_segments<T><<<1024, TPB, 0, st>>>(d, kp);
  k_sort_gather<T><<<1024, TPB, 0, st>>>(d, kp);
  LAUNCH_COUNT(); LAUNCH_COUNT(); LAUNCH_COUNT(); LAUNCH_COUNT();
  Particles<T> t = d.p; d.p = d.p2; d.p2 = t;
  uint16_t* o = d.owner; d.owner = d.owner2; d.owner2 = o;
  uint8_t* c = d.inc; d.inc = d.inc2; d.inc2 = c;
  // slot q now holds the particle the reference numbers q
  if (d.lid) { d.lid2 = d.lid; d.lid = nullptr; d.lpos = nullptr; }
}

// --------------------------------------------------------------- reductions --
template <typename T>
__global__ void k_observables(Dev<T> d, KParams<T> kp, double m0, double m1, double m2, double m3) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (sizeof(T) == 4) {
    // FP32 build: compensated (Kahan) FP32 sums per thread, widened to FP64
    // for the reduction over threads; FP64 arithmetic per particle would run
    // at the part's FP64 rate
    const float mf0 = (float)m0, mf1 = (float)m1, mf2 = (float)m2, mf3 = (float)m3;
    float sum[4] = {0.f, 0.f, 0.f, 0.f}, cmp[4] = {0.f, 0.f, 0.f, 0.f};
    uint32_t cnt[4] = {0u, 0u, 0u, 0u};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) {
      const uint8_t f = d.p.flag[i];
      float vx, vy, vz;
      int sp;
      if (f & FLAG_HOME_SHELL) {
        const uint32_t j = d.p.cell[i];
        vx = (float)d.sh.vx[j]; vy = (float)d.sh.vy[j]; vz = (float)d.sh.vz[j];
        sp = d.sh.flag[j] & FLAG_SPECIES;
      } else {
        vx = (float)d.p.vx[i]; vy = (float)d.p.vy[i]; vz = (float)d.p.vz[i];
        sp = f & FLAG_SPECIES;
      }
      const float m = sp == 0 ? mf0 : (sp == 1 ? mf1 : (sp == 2 ? mf2 : mf3));
      const float term[4] = {m * vx, m * vy, m * vz, 0.5f * m * (vx * vx + vy * vy + vz * vz)};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float y = term[k] - cmp[k];
        const float t = sum[k] + y;
        cmp[k] = (t - sum[k]) - y;
        sum[k] = t;
      }
      cnt[0] += sp == 0; cnt[1] += sp == 1; cnt[2] += sp == 2; cnt[3] += sp == 3;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      double v = k < 4 ? widen_f32(sum[k]) - widen_f32(cmp[k]) : (double)cnt[k - 4];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if ((threadIdx.x & 31) == 0) atomicAdd(&d.ctr->sums[k], v);
    }
    return;
  }
  const double mass[4] = {m0, m1, m2, m3};
  double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) {
    uint8_t f = d.p.flag[i];
    double vx, vy, vz;
    int sp;
    if (f & FLAG_HOME_SHELL) {
      uint32_t j = d.p.cell[i];
      vx = d.sh.vx[j]; vy = d.sh.vy[j]; vz = d.sh.vz[j];
      sp = d.sh.flag[j] & FLAG_SPECIES;
    } else {
      vx = d.p.vx[i]; vy = d.p.vy[i]; vz = d.p.vz[i];
      sp = f & FLAG_SPECIES;
    }
    double m = mass[sp];
    s[0] += m * vx; s[1] += m * vy; s[2] += m * vz;
    s[3] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
    s[4 + sp] += 1.0;
  }
  for (int k = 0; k < 8; ++k) {
    double v = s[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&d.ctr->sums[k], v);
  }
}

template <typename T>
void Launch<T>::observables(const Dev<T>& d, const KParams<T>& kp, const double* mass, int grid, cudaStream_t st) {
  k_observables<T><<<grid, TPB, 0, st>>>(d, kp, mass[0], mass[1], mass[2], mass[3]);
  LAUNCH_COUNT();
}

// ------------------------------------------------------------------ init ----
// initial_mod.f95:122-345 with contract draws: rejection sampling of the
// positions against the sphere cutoffs and Box-Muller velocities (cos branch,
// gauss_rand_mod.f95:31-39).  The mean removal runs on the host afterwards.
template <typename T>
__global__ void k_init_solvent(Dev<T> d, KParams<T> kp, int64_t b0, int64_t b1, int64_t b2,
                               double v0, double v1, double v2, double v3) {
  const double sd[4] = {v0, v1, v2, v3};
  const double pi = 3.141592653589793;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) {
    int code = i < b0 ? 0 : (i < b1 ? 1 : (i < b2 ? 2 : 3));
    bool ok = false;
    uint32_t cell = 0;
    T ox = 0, oy = 0, oz = 0;
    for (uint32_t at = 0; at < 1000000u && !ok; ++at) {
      double ux, uy, uz, un;
      contract_pair(kp.seed, TAG_INIT_POS, (uint32_t)i, at, 0, ux, uy);
      contract_pair(kp.seed, TAG_INIT_POS, (uint32_t)i, at, 1, uz, un);
      double X = kp.Ld[0] * ux, Y = kp.Ld[1] * uy, Z = kp.Ld[2] * uz;
      double fx = floor(X), fy = floor(Y), fz = floor(Z);
      int cx = min((int)fx, kp.lx - 1), cy = min((int)fy, kp.ly - 1), cz = min((int)fz, kp.lz - 1);
      cell = pack_cell(cx, cy, cz);
      ox = (T)(X - cx); oy = (T)(Y - cy); oz = (T)(Z - cz);
      ok = true;
      if (kp.ns > 0) {
        int bin = bin_of(kp.lx, kp.ly, kp.nbx, kp.nby, cell);
        unsigned int nc = d.bin_cnt[bin];
        const uint16_t* bl = d.bin_list + (size_t)bin * BIN_SLOTS;
        for (unsigned int q = 0; q < nc && ok; ++q) {
          int s = bl[q];
          double dx = X - d.dpos[3 * s], dy = Y - d.dpos[3 * s + 1], dz = Z - d.dpos[3 * s + 2];
          dx = dmin_image(dx, kp.Ld[0]);
          dy = dmin_image(dy, kp.Ld[1]);
          if (kp.geometry == 1) dz = dmin_image(dz, kp.Ld[2]);
          if (dx * dx + dy * dy + dz * dz < (double)kp.cut2_strict[s & 1]) ok = false;
        }
      }
    }
    if (!ok) atomicOr(&d.ctr->status, DEV_ERR_INIT);
    d.p.cell[i] = cell;
    d.p.ox[i] = ox; d.p.oy[i] = oy; d.p.oz[i] = oz;
    d.p.flag[i] = (uint8_t)code;
    T* vv[3] = {d.p.vx, d.p.vy, d.p.vz};
    for (int comp = 0; comp < 3; ++comp) {
      double xx, yy;
      contract_pair(kp.seed, TAG_INIT_VEL, (uint32_t)i, (uint32_t)comp, 0, xx, yy);
      yy = 1.0 - yy;
      double th = 2 * pi * xx, R = sqrt(-2 * log(yy));
      vv[comp][i] = (T)(sd[code] * (R * cos(th)) + 0.0);
    }
  }
}

template <typename T>
__global__ void k_sum_vel(Dev<T> d, KParams<T> kp) {
  double s[3] = {0, 0, 0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) {
    s[0] += (double)d.p.vx[i]; s[1] += (double)d.p.vy[i]; s[2] += (double)d.p.vz[i];
  }
  for (int k = 0; k < 3; ++k) {
    double v = s[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&d.ctr->sums[8 + k], v);
  }
}

template <typename T>
__global__ void k_sub_mean(Dev<T> d, KParams<T> kp) {
  const double inv = 1.0 / (double)kp.n;
  const double mx = d.ctr->sums[8] * inv, my = d.ctr->sums[9] * inv, mz = d.ctr->sums[10] * inv;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < kp.n; i += stride) {
    T* vv[3] = {d.p.vx, d.p.vy, d.p.vz};
    const double m[3] = {mx, my, mz};
    for (int c = 0; c < 3; ++c) {
      const double w = (double)vv[c][i] - m[c];
      if (sizeof(T) == 8) { vv[c][i] = (T)w; continue; }
      // FP32: the drawn velocities lie on the float grid and the mean is one
      // constant, so round-to-nearest would give every velocity of a binade
      // the same error and leave a net momentum of order N ulp.  Round up or
      // down at random instead (probability = distance to the other
      // neighbour over the spacing), from a contract draw of the particle:
      // unbiased and independent, the residual is a random walk of order
      // sqrt(N) ulp.
      float f = (float)w;
      const double r = w - (double)f;
      if (r != 0.0) {
        const float g = nextafterf(f, r > 0.0 ? INFINITY : -INFINITY);
        double u, unused;
        contract_pair(kp.seed, TAG_INIT_VEL, (uint32_t)i, (uint32_t)(4 + c), 0, u, unused);
        if (u * ((double)g - (double)f) * (r > 0.0 ? 1.0 : -1.0) < fabs(r)) f = g;
      }
      vv[c][i] = (T)f;
    }
  }
}

template <typename T>
void Launch<T>::init_solvent(const Dev<T>& d, const KParams<T>& kp, const int64_t* bounds, double kT,
                             const double* mass, cudaStream_t st) {
  double sd[4];
  for (int c = 0; c < 4; ++c) sd[c] = sqrt(kT / mass[c]);
  k_init_solvent<T><<<1024, TPB, 0, st>>>(d, kp, bounds[0], bounds[1], bounds[2], sd[0], sd[1], sd[2], sd[3]);
  cudaMemsetAsync(&d.ctr->sums[8], 0, 3 * sizeof(double), st);
  k_sum_vel<T><<<512, TPB, 0, st>>>(d, kp);
  k_sub_mean<T><<<1024, TPB, 0, st>>>(d, kp);
  LAUNCH_COUNT(); LAUNCH_COUNT(); LAUNCH_COUNT();
}


}  // namespace mpcmd
