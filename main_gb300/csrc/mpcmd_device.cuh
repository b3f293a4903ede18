// Device-side building blocks of the mpcmd engine (sm_103a).
//
// Particle layout (structure of arrays, resident in HBM):
//   cell  u32   packed cell coordinates ix | iy << 10 | iz << 20 (box edges <= 1024)
//   ox..  T     offset inside the cell, [0, 1)  (T = float in production, double for parity)
//   vx..  T     velocity
//   flag  u8    bits 0-1 species code, bit 3 state written at the last rebuild (else at
//               the last full pass: rebuilds between collision steps leave far particles
//               unwritten and their lazy stream deferred), bit 4 member of the shell ("inside") list that
//               flies freely until the next collision and is streamed lazily like an
//               outside particle, bit 5 member of the shell list of the last rebuild whose
//               state is current, bit 6 state lives in the shell buffer (then cell[] holds
//               the shell slot)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define MPCMD_HD __host__ __device__ __forceinline__

namespace mpcmd {

enum Tag : uint32_t {
  TAG_SHIFT = 1, TAG_AXIS = 2, TAG_RXN = 3, TAG_CAT = 4,
  TAG_INIT_DIMER = 5, TAG_INIT_POS = 6, TAG_INIT_VEL = 7
};

constexpr uint8_t FLAG_SPECIES = 0x03;
constexpr uint8_t FLAG_FRESH = 0x08;     // main-home state is at the last rebuild, not the last full pass
constexpr uint8_t FLAG_PASSIVE = 0x10;   // shell member in free flight, kept in the main home
constexpr uint8_t FLAG_INLIST = 0x20;
constexpr uint8_t FLAG_HOME_SHELL = 0x40;
constexpr int PAIRMAX = 8;         // spheres one shell particle may interact with
constexpr int BIN_SLOTS = 16;      // spheres one coarse bin may list
constexpr int BIN_EDGE = 4;        // coarse bin edge in cells
constexpr int GAP_EDGE = 2;        // gap-field bin edge in cells (watch list)

// ---------------------------------------------------------------- Philox --
// Philox4x32-10 (Salmon et al., SC'11): counter (index, extra, step, tag),
// key = 64-bit seed.
MPCMD_HD void philox4x32_10(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3,
                            uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
  }
}

MPCMD_HD double u01_53(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)a << 21) | (uint64_t)(b >> 11);
  return (double)m * (1.0 / 9007199254740992.0);
}

// Both doubles of one counter: u[0] from words 0,1 and u[1] from words 2,3.
MPCMD_HD void contract_pair(uint64_t seed, uint32_t tag, uint32_t index, uint32_t extra,
                            uint32_t step, double& u0, double& u1) {
  uint32_t c0 = index, c1 = extra, c2 = step, c3 = tag;
  philox4x32_10(c0, c1, c2, c3, (uint32_t)seed, (uint32_t)(seed >> 32));
  u0 = u01_53(c0, c1);
  u1 = u01_53(c2, c3);
}

// The two 53-bit mantissas as integers (for FP64-free comparisons).
MPCMD_HD void contract_bits(uint64_t seed, uint32_t tag, uint32_t index, uint32_t extra,
                            uint32_t step, uint64_t& m0, uint64_t& m1) {
  uint32_t c0 = index, c1 = extra, c2 = step, c3 = tag;
  philox4x32_10(c0, c1, c2, c3, (uint32_t)seed, (uint32_t)(seed >> 32));
  m0 = ((uint64_t)c0 << 21) | (uint64_t)(c1 >> 11);
  m1 = ((uint64_t)c2 << 21) | (uint64_t)(c3 >> 11);
}

// Leading 32-bit words of both draws of one counter (one Philox evaluation):
// w0 the top bits of contract_pair's u0, w2 those of u1.
MPCMD_HD void contract_words(uint64_t seed, uint32_t tag, uint32_t index, uint32_t extra,
                             uint32_t step, uint32_t& w0, uint32_t& w2) {
  uint32_t c0 = index, c1 = extra, c2 = step, c3 = tag;
  philox4x32_10(c0, c1, c2, c3, (uint32_t)seed, (uint32_t)(seed >> 32));
  w0 = c0;
  w2 = c2;
}

// Integer threshold of a probability p for draws compared as `p > u`:
// p > m / 2^53  <=>  m < ceil(p 2^53)  (m the 53-bit mantissa).
inline uint64_t prob_threshold(double p) {
  if (!(p > 0.0)) return 0ull;
  if (p >= 1.0) return 1ull << 53;
  return (uint64_t)ceil(p * 9007199254740992.0);
}

// ------------------------------------------------------------- cells ------
MPCMD_HD uint32_t pack_cell(int x, int y, int z) {
  return (uint32_t)x | ((uint32_t)y << 10) | ((uint32_t)z << 20);
}
MPCMD_HD int cell_x(uint32_t c) { return (int)(c & 1023u); }
MPCMD_HD int cell_y(uint32_t c) { return (int)((c >> 10) & 1023u); }
MPCMD_HD int cell_z(uint32_t c) { return (int)(c >> 20); }

// Scalars every kernel needs, in the working precision T and in FP64.
template <typename T>
struct KParams {
  int lx, ly, lz;
  int geometry;          // 0 walls, 1 periodic
  int ns, nd;
  int catalysis, exclusion, kinetics, rotation_sense;
  int react_dir;
  int cell_capacity;
  int64_t n;             // solvent particles
  int64_t ncell, ncell_shift;
  uint64_t seed;
  T Lx, Ly, Lz;
  T dt;
  T hIM[4];              // (0.5 dt)/m per species code
  T eps_c[4], eps_n[4];
  T cut2[2], full2[2];   // LJ cutoff^2 and (cutoff + skin)^2, [0] C, [1] N
  T R6[2], R12[2], r6R6[2], r12R12[2];
  T msd_thr;             // (0.5 skin)^2
  T cosrot, sinrot;
  double rp_ab, rp_ba;
  uint64_t thr_ab, thr_ba;   // integer thresholds of rp_ab / rp_ba on the 53-bit draws
  double tau;            // MPC interval
  double k[6];
  float kf[6], tauf;      // the same rounded to float (FP32 reaction path)
  double dtd;            // MD step in FP64
  int nbx, nby, nbz;     // coarse sphere-bin grid
  int ngx, ngy, ngz;     // gap-field grid (GAP_EDGE cells per bin edge)
  // dimer constants (FP64): sphere-sphere LJ by pair type [CC, CN, NN]
  double Ld[3];
  double mot_cut2[3], mot_R6[3], mot_R12[3], mot_r6R6[3], mot_r12R12[3];
  float mot_cut2f[3];
  double em, ew, rwc, rwn;
  int rotor;             // anchored dimers, harmonic z tether, no motor-motor LJ
  int owner_tags;        // B particles tagged with the motor that made them (type_B)
  double tether_k, tether_z;
  double mc, mn, dcn;
  // dimer constants, computed once on the host with the kernel's expressions
  double hIMc, hIMn, IIM;          // (dt/2)/Mc, (dt/2)/Mn, 1/(1/Mc + 1/Mn)
  double iMc, iMn, iD2, iMcdt, iMndt;   // 1/Mc, 1/Mn, 1/Dcn^2, 1/(Mc dt), 1/(Mn dt)
  T cut2_strict[2];      // (R * 2^(1/6))^2 for the initial placement test
};

// Sphere position as cell + offset in T (written whenever a sphere moves).
template <typename T>
struct SphereRel {
  int cx, cy, cz;
  T ox, oy, oz;
};

template <typename T>
MPCMD_HD T min_image(T d, T L) {
  if (d > (T)0.5 * L) d -= L;
  else if (d < -(T)0.5 * L) d += L;
  return d;
}

template <typename T>
__device__ __forceinline__ T tfloor(T x);
template <>
__device__ __forceinline__ float tfloor<float>(float x) { return floorf(x); }
template <>
__device__ __forceinline__ double tfloor<double>(double x) { return floor(x); }

// Offset renormalisation: fold the integer part of o into the cell index.
template <typename T>
__device__ __forceinline__ void renorm(T& o, int& c) {
  T f = tfloor(o);
  o -= f;
  c += (int)f;
  if (o >= (T)1) { o -= (T)1; c += 1; }
}

// Periodic wrap of a cell coordinate.  For moves shorter than the box this is
// the single shift of evolve_mod.f95:260-264; longer moves (which the Fortran
// does not handle) still land inside the box, so no index leaves its table.
__device__ __forceinline__ int wrap_cell(int c, int L) {
  if (c >= L) c -= L;
  else if (c < 0) c += L;
  if (c >= L || c < 0) { c %= L; if (c < 0) c += L; }
  return c;
}

// Separation solvent - sphere with the geometry's minimum image.
template <typename T>
__device__ __forceinline__ T sep2(const KParams<T>& kp, uint32_t cell, T ox, T oy, T oz,
                                  const SphereRel<T>& s, T& dx, T& dy, T& dz) {
  dx = (T)(cell_x(cell) - s.cx) + (ox - s.ox);
  dy = (T)(cell_y(cell) - s.cy) + (oy - s.oy);
  dz = (T)(cell_z(cell) - s.cz) + (oz - s.oz);
  dx = min_image(dx, kp.Lx);
  dy = min_image(dy, kp.Ly);
  if (kp.geometry == 1) dz = min_image(dz, kp.Lz);
  return dx * dx + dy * dy + dz * dz;
}

// Free flight of one particle over d = v*dt (or (v*dt)*tc for the lazy
// streaming of outside particles), with the x/y periodic wrap, the z
// bounce-back walls and the reactive floor (evolve_mod.f95:258-314, :473-527,
// reactive_grid_mod.f95:103-151), or the fully periodic box.
template <typename T>
__device__ __forceinline__ void stream_one(const KParams<T>& kp, const uint8_t* react_box,
                                           uint32_t& cell, T& ox, T& oy, T& oz,
                                           T& vx, T& vy, T& vz, uint8_t& flag,
                                           bool lazy, int tc) {
  int cx = cell_x(cell), cy = cell_y(cell), cz = cell_z(cell);
  T ddx = vx * kp.dt, ddy = vy * kp.dt, ddz = vz * kp.dt;
  if (lazy) { ddx = ddx * (T)tc; ddy = ddy * (T)tc; ddz = ddz * (T)tc; }
  ox = ox + ddx; renorm(ox, cx); cx = wrap_cell(cx, kp.lx);
  oy = oy + ddy; renorm(oy, cy); cy = wrap_cell(cy, kp.ly);
  oz = oz + ddz;
  if (kp.geometry == 0) {
    T zlo = (T)cz + oz;               // absolute z
    T zhi = (T)(cz - kp.lz) + oz;     // z - Lz
    bool bounce = false;
    T t = (T)0;
    if (zlo < (T)0) {
      t = zlo / vz;
      // reactive floor: back-project to the hit point (x, y after the wrap)
      T ax = ox - vx * t, ay = oy - vy * t;
      int hx = cx, hy = cy;
      renorm(ax, hx); hx = wrap_cell(hx, kp.lx);
      renorm(ay, hy); hy = wrap_cell(hy, kp.ly);
      if (react_box[hx + kp.lx * hy]) {
        uint8_t sp = flag & FLAG_SPECIES;
        if (kp.react_dir == 0 && sp == 0) flag = (flag & ~FLAG_SPECIES) | 1;
        else if (kp.react_dir == 1 && sp == 1) flag = (flag & ~FLAG_SPECIES) | 0;
      }
      bounce = true;
    } else if (zhi > (T)0) {
      t = zhi / vz;
      bounce = true;
    }
    if (bounce) {
      vx = (T)-1 * vx; vy = (T)-1 * vy; vz = (T)-1 * vz;
      ox = ox + (T)2 * vx * t; renorm(ox, cx); cx = wrap_cell(cx, kp.lx);
      oy = oy + (T)2 * vy * t; renorm(oy, cy); cy = wrap_cell(cy, kp.ly);
      oz = oz + (T)2 * vz * t;
    }
    renorm(oz, cz);
    if (cz >= kp.lz) { cz = kp.lz - 1; oz = (T)1; }   // exactly on the upper wall
    if (cz < 0) { cz = 0; oz = (T)0; }
  } else {
    renorm(oz, cz);
    cz = wrap_cell(cz, kp.lz);
  }
  cell = pack_cell(cx, cy, cz);
}

// Shifted collision cell (mpc_rotation_mod.f95:110-148 / RMPC:31-46), 0-based.
template <typename T>
__device__ __forceinline__ uint32_t shifted_key(const KParams<T>& kp, uint32_t cell,
                                                T ox, T oy, T oz, T sx, T sy, T sz) {
  int cx = cell_x(cell), cy = cell_y(cell), cz = cell_z(cell);
  int fx = cx + (int)tfloor(ox + sx);
  int fy = cy + (int)tfloor(oy + sy);
  fx = wrap_cell(fx, kp.lx);
  fy = wrap_cell(fy, kp.ly);
  int fz;
  if (kp.geometry == 0) {
    fz = cz + (int)tfloor(sz < (T)0 ? (oz + sz) + (T)1 : oz + sz);
  } else {
    fz = wrap_cell(cz + (int)tfloor(oz + sz), kp.lz);
  }
  return (uint32_t)fx + (uint32_t)kp.lx * ((uint32_t)fy + (uint32_t)kp.ly * (uint32_t)fz);
}

__device__ __forceinline__ uint32_t unshifted_id(int lx, int ly, uint32_t cell) {
  return (uint32_t)cell_x(cell) + (uint32_t)lx * ((uint32_t)cell_y(cell) + (uint32_t)ly * (uint32_t)cell_z(cell));
}

// Ordered-integer image of a non-negative float/double for atomicMax.
__device__ __forceinline__ unsigned int ord_bits(float v) { return __float_as_uint(v); }
__device__ __forceinline__ unsigned long long ord_bits(double v) {
  return (unsigned long long)__double_as_longlong(v);
}

// Exact widening of a binary32 value to binary64 by rearranging its IEEE-754
// fields in integer registers: the same value as (double)f for every normal
// number, zero, infinity and NaN; subnormal floats (|f| < 2^-126) become a
// signed zero.  On GB300 the conversion instruction runs on the FP64 pipe,
// about 16 SM cycles per warp, which the per-sphere force sums would pay
// several times per warp; this form uses the integer pipes only.
__device__ __forceinline__ double widen_f32(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t sign = u & 0x80000000u;
  const uint32_t e = (u >> 23) & 0xFFu;
  const uint32_t m = u & 0x007FFFFFu;
  uint32_t hi, lo;
  if (e == 0u) {            // zero (and subnormals)
    hi = sign; lo = 0u;
  } else if (e == 0xFFu) {  // infinity / NaN keep their class
    hi = sign | 0x7FF00000u | (m >> 3); lo = m << 29;
  } else {                  // rebias the exponent 127 -> 1023
    hi = sign | ((e + 896u) << 20) | (m >> 3); lo = m << 29;
  }
  return __hiloint2double((int)hi, (int)lo);
}
__device__ __forceinline__ double to_f64(float f) { return widen_f32(f); }
__device__ __forceinline__ double to_f64(double f) { return f; }

}  // namespace mpcmd
