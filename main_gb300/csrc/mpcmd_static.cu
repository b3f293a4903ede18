// mpcmd_collide_static: the SRD collision of a caller-owned particle set with
// no device allocation at all.
//
// Who needs it: callers that cannot call cudaMalloc.  A Fortran or C host that
// embeds this library inside a larger code whose memory manager owns every
// byte of device memory (a pool sized at start-up, or a framework allocator)
// may not allocate behind that manager's back; and a caller in a tight
// stepping loop cannot afford cudaMalloc/cudaFree, which synchronise the
// device.  The context API (mpcmd_create) allocates its whole state up front,
// so those callers use this entry point instead: they pass device arrays they
// already own, and the only scratch memory is the file-scope array below.
//
// Scratch: g_collide_scratch, a static __device__ array of
// MPCMD_STATIC_MAX_CELLS x 4 doubles (16 MiB).  Every GPU that loads this
// library holds it until the process exits.  Every call on a device shares it
// and it keeps the last call's contents, so each call clears the part it uses
// before accumulating; calls that overlap on the GPU (different streams or
// host threads, same device) race on it and must be serialised by the caller.
//
// Set-up: the first call on each device (with that device current) resolves
// the array's device address with cudaGetSymbolAddress, which also loads this
// module on the device.  Make that first call before any stream capture.  A
// call on a stream that is not capturing resolves the address again (a host
// lookup, no allocation), so after cudaDeviceReset the next uncaptured call
// picks up the reloaded module's array; a captured call uses the address of
// the last uncaptured one.
//
// The arithmetic is the FP64 collision stage of the engine (k_accumulate_main,
// k_cells and k_rotate_main in mpcmd_kernels.cuh; mpc_rotation_mod.f95:102-228
// and RMPC_SelkovDimer.f90:15-120 in the reference), fused into a clear, an
// accumulate and a rotate kernel; the centre of mass and the axis are derived
// from the sums in the rotate pass instead of a per-cell table.
#include <algorithm>
#include <cmath>
#include <mutex>

#include "mpcmd.h"
#include "mpcmd_kernels.cuh"   // rotate_v and the device helpers

using namespace mpcmd;

namespace {

constexpr int64_t kMaxCells = MPCMD_STATIC_MAX_CELLS;
constexpr int kMaxDevices = 64;
constexpr int kThreads = 256;

// count, sum vx, sum vy, sum vz of each shifted cell
static __device__ __align__(256) double g_collide_scratch[4 * kMaxCells];

std::mutex g_setup_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// Cell and in-cell offset of one absolute coordinate, as the engine's upload
// conversion computes them (k_upload_pos).
__device__ __forceinline__ void to_cell(double x, int L, bool wrap, int& c, double& o) {
  double f = floor(x);
  c = (int)f;
  o = x - f;
  if (o >= 1.0) { o -= 1.0; c += 1; }
  if (wrap) {
    c = wrap_cell(c, L);
  } else {
    if (c >= L) { c = L - 1; o = 1.0; }
    if (c < 0) { c = 0; o = 0.0; }
  }
}

__device__ __forceinline__ uint32_t static_key(const KParams<double>& kp, double x, double y, double z,
                                               double sx, double sy, double sz) {
  int cx, cy, cz;
  double ox, oy, oz;
  to_cell(x, kp.lx, true, cx, ox);
  to_cell(y, kp.ly, true, cy, oy);
  to_cell(z, kp.lz, kp.geometry == MPCMD_GEOM_PERIODIC, cz, oz);
  return shifted_key(kp, pack_cell(cx, cy, cz), ox, oy, oz, sx, sy, sz);
}

__global__ void k_static_clear(double* acc, int64_t nwords) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nwords; i += stride) acc[i] = 0.0;
}

__global__ void k_static_accumulate(KParams<double> kp, const double* x, const double* y, const double* z,
                                    const double* vx, const double* vy, const double* vz, int64_t n,
                                    double sx, double sy, double sz, double* acc) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    uint32_t key = static_key(kp, x[i], y[i], z[i], sx, sy, sz);
    if ((int64_t)key >= kp.ncell_shift) continue;   // defensive: keys are in range by construction
    double* a = acc + 4 * (size_t)key;
    atomicAdd(a + 0, 1.0);
    atomicAdd(a + 1, vx[i]);
    atomicAdd(a + 2, vy[i]);
    atomicAdd(a + 3, vz[i]);
  }
}

__global__ void k_static_rotate(KParams<double> kp, const double* x, const double* y, const double* z,
                                double* vx, double* vy, double* vz, int64_t n, double sx, double sy,
                                double sz, uint32_t step, const double* acc) {
  const double pi = 3.141592653589793;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    uint32_t key = static_key(kp, x[i], y[i], z[i], sx, sy, sz);
    if ((int64_t)key >= kp.ncell_shift) continue;
    const double* a = acc + 4 * (size_t)key;
    const double cnt = a[0];
    double r[6];
    if (kp.rotation_sense > 0) {
      r[0] = a[1] / cnt; r[1] = a[2] / cnt; r[2] = a[3] / cnt;
    } else {
      const double inv = 1.0 / cnt;
      r[0] = a[1] * inv; r[1] = a[2] * inv; r[2] = a[3] * inv;
    }
    double u1, u2;
    contract_pair(kp.seed, TAG_AXIS, key, 0, step, u1, u2);
    const double phi = 2.0 * pi * u1, theta = 2.0 * u2 - 1.0;
    r[3] = sqrt(1.0 - theta * theta) * cos(phi);
    r[4] = sqrt(1.0 - theta * theta) * sin(phi);
    r[5] = theta;
    double wx = vx[i], wy = vy[i], wz = vz[i];
    rotate_v(kp, r, wx, wy, wz);
    vx[i] = wx; vy[i] = wy; vz[i] = wz;
  }
}

}  // namespace

extern "C" int mpcmd_collide_static(const double* x, const double* y, const double* z, double* vx,
                                    double* vy, double* vz, int64_t n, int32_t lx, int32_t ly,
                                    int32_t lz, int32_t geometry, double rot_angle,
                                    int32_t rotation_sense, uint64_t seed, int64_t step,
                                    void* stream) {
  // An error the calling thread left pending is its own: report it without
  // launching and leave it in place for the caller's cudaGetLastError.
  if (cudaPeekAtLastError() != cudaSuccess) return MPCMD_ERR_CUDA;
  if (n < 0 || lx <= 0 || ly <= 0 || lz <= 0 || lx > 1024 || ly > 1024 || lz > 1024) return MPCMD_ERR_CONFIG;
  if (geometry != MPCMD_GEOM_WALLS && geometry != MPCMD_GEOM_PERIODIC) return MPCMD_ERR_CONFIG;
  if (rotation_sense != 1 && rotation_sense != -1) return MPCMD_ERR_CONFIG;
  const int64_t ncs = (int64_t)lx * ly * (geometry == MPCMD_GEOM_WALLS ? (int64_t)lz + 1 : (int64_t)lz);
  if (ncs > kMaxCells) return MPCMD_ERR_CONFIG;   // beyond the static scratch array
  if (n > 0 && (!x || !y || !z || !vx || !vy || !vz)) return MPCMD_ERR_CONFIG;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MPCMD_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return MPCMD_ERR_CONFIG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) return MPCMD_ERR_CUDA;
  double* acc = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev] || cap == cudaStreamCaptureStatusNone) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_collide_scratch) != cudaSuccess || !p) return MPCMD_ERR_CUDA;
      g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    acc = g_scratch_ptr[dev];
  }
  if (n == 0) return MPCMD_OK;

  KParams<double> kp{};
  kp.lx = lx; kp.ly = ly; kp.lz = lz;
  kp.geometry = geometry;
  kp.rotation_sense = rotation_sense;
  kp.ncell_shift = ncs;
  kp.seed = seed;
  kp.cosrot = std::cos(rot_angle);
  kp.sinrot = std::sin(rot_angle);
  // grid shift: the contract stream (SHIFT, 0, extra, step) as the engine draws it
  double u0, u1, u2, u3;
  contract_pair(seed, TAG_SHIFT, 0, 0, (uint32_t)step, u0, u1);
  contract_pair(seed, TAG_SHIFT, 0, 1, (uint32_t)step, u2, u3);
  const double sx = u0 - 0.5, sy = u1 - 0.5, sz = u2 - 0.5;

  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return MPCMD_ERR_CUDA;
  const int64_t want = (n + kThreads - 1) / kThreads;
  const int grid = (int)std::min<int64_t>(want, (int64_t)nsm * 8);
  const int cgrid = (int)std::min<int64_t>((4 * ncs + kThreads - 1) / kThreads, (int64_t)nsm * 8);
  k_static_clear<<<cgrid, kThreads, 0, st>>>(acc, 4 * ncs);
  k_static_accumulate<<<grid, kThreads, 0, st>>>(kp, x, y, z, vx, vy, vz, n, sx, sy, sz, acc);
  k_static_rotate<<<grid, kThreads, 0, st>>>(kp, x, y, z, vx, vy, vz, n, sx, sy, sz, (uint32_t)step, acc);
  if (cudaPeekAtLastError() != cudaSuccess) return MPCMD_ERR_CUDA;
  return MPCMD_OK;
}
