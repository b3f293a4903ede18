// Exclusive u32 prefix sum and the launch counter shared by both precisions.
#include <cstdio>
#include "mpcmd_engine.cuh"

namespace mpcmd {

int64_t g_kernel_launches = 0;

// Checked builds synchronise after every launch and name the failing launcher.
int debug_sync(cudaStream_t st, const char* where, int line) {
  cudaError_t e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) std::fprintf(stderr, "mpcmd checked build: %s:%d: %s\n", where, line, cudaGetErrorString(e));
  return 0;
}

#ifdef MPCMD_CHECKED
#define LAUNCH_COUNT() (++g_kernel_launches, debug_sync(st, __func__, __LINE__))
#else
#define LAUNCH_COUNT() (++g_kernel_launches)
#endif

// ------------------------------------------------------------------ scan ----
// Exclusive prefix sum of u32 (three-phase: tile sums, scan of tile sums,
// tile scan with offsets).  Tile = 4 * TPB elements.
constexpr int SCAN_TILE = 4 * TPB;

__global__ void k_scan_tiles(const uint32_t* in, int64_t n, uint32_t* tile_sums) {
  __shared__ uint32_t sh[TPB / 32];
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  uint32_t s = 0;
  for (int k = 0; k < 4; ++k) {
    int64_t i = base + (int64_t)k * TPB + threadIdx.x;
    if (i < n) s += in[i];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < TPB / 32; ++w) t += sh[w];
    tile_sums[blockIdx.x] = t;
  }
}

__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t ws[TPB / 32];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t t = lane < TPB / 32 ? ws[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < TPB / 32) ws[lane] = t;
  }
  __syncthreads();
  uint32_t pre = (w > 0 ? ws[w - 1] : 0) + x - v;
  if (total) *total = ws[TPB / 32 - 1];
  __syncthreads();
  return pre;
}

__global__ void k_scan_apply(const uint32_t* in, uint32_t* out, int64_t n, const uint32_t* tile_offsets) {
  int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
  uint32_t carry = tile_offsets[blockIdx.x];
  for (int k = 0; k < 4; ++k) {
    int64_t i = base + (int64_t)k * TPB + threadIdx.x;
    uint32_t v = i < n ? in[i] : 0;
    uint32_t tot;
    uint32_t pre = block_exclusive_scan(v, &tot);
    if (i < n) out[i] = carry + pre;
    carry += tot;
  }
}

int64_t scan_tmp_words(int64_t n) {
  int64_t words = 0;
  while (n > 1) {
    int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    words += 2 * tiles + 8;
    n = tiles;
  }
  return words + 16;
}

void scan_u32(const uint32_t* in, uint32_t* out, int64_t n, uint32_t* tmp, cudaStream_t st) {
  int64_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (tiles <= 1) {
    cudaMemsetAsync(tmp, 0, sizeof(uint32_t), st);
    k_scan_apply<<<1, TPB, 0, st>>>(in, out, n, tmp);
    LAUNCH_COUNT();
    return;
  }
  uint32_t* sums = tmp;
  uint32_t* offs = tmp + tiles + 4;
  k_scan_tiles<<<(unsigned)tiles, TPB, 0, st>>>(in, n, sums);
  LAUNCH_COUNT();
  scan_u32(sums, offs, tiles, offs + tiles + 4, st);
  k_scan_apply<<<(unsigned)tiles, TPB, 0, st>>>(in, out, n, offs);
  LAUNCH_COUNT();
}

}  // namespace mpcmd
