// Learned surrogate of the batched ensemble: a multilayer perceptron
// (n_in inputs -> n_layers hidden layers of width H with SiLU -> n_out
// outputs) trained and evaluated by this file's own kernels on the
// fifth-generation tensor cores of sm_103a.
//
// Every contraction (forward, input gradient, weight gradient) is one GEMM
// form, C[M, N] = A[M, K] . B[N, K]^T with A and B BF16 and K-major, and one
// persistent kernel, k_gemm, with one CTA per SM walking its share of the
// 128 x BN output tiles.  Warp roles: one thread streams the A and B tiles
// into a ring of shared-memory stages with TMA (cp.async.bulk.tensor,
// 128-byte swizzle, mbarriers), or keeps B resident when all of it fits one
// tile (the hidden layers of inference); one thread issues tcgen05.mma
// (kind::f16, BF16 operands, FP32 accumulator in tensor memory) and releases
// each stage with tcgen05.commit; sixteen epilogue warps read the
// accumulator back with tcgen05.ld (a warp reaches the 32 TMEM lanes of its
// quarter; the four warps of a quarter take its 32-column chunks in turn)
// and apply the fused epilogue: bias + SiLU with the pre-activation kept for
// the backward pass (forward hidden), bias + SiLU (inference), bias
// (output), SiLU' of the kept pre-activation (input gradient), or the FP32
// weight gradient.  Two accumulators in tensor memory let the epilogue of
// one tile overlap the loads and MMAs of the next.  Row-major outputs go
// through a per-warp 32-row staging tile in shared memory so that every
// store writes whole rows; the forms that the next GEMM needs transposed are
// written from the thread-per-row layout, so that every operand stays
// K-major.  Every mbarrier wait is bounded (two seconds of globaltimer): on
// expiry the kernel raises an error flag, skips its remaining work, waits
// for its copies and MMAs in flight and still frees its tensor memory.
//
// Weights are kept in FP32 (master copy for Adam) and in BF16 twice: [N, K]
// for the forward GEMM and [K, N] for the input-gradient GEMM.
#include <cuda.h>   // CUtensorMap and the encoder's signature (resolved at run time)
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "mpcmd.h"

namespace {

constexpr int BM = 128;        // output rows per tile (the MMA's M)
constexpr int BK = 64;         // K per stage: one 128-byte swizzle row of BF16
constexpr int EPI_WARPS = 16;                 // four per TMEM lane quarter
constexpr int THREADS = 64 + 32 * EPI_WARPS;   // producer warp, MMA warp, epilogue warps
constexpr int A_STAGE = BM * BK * 2;   // 16 KiB
constexpr int K_MAX = 256;             // the longest K (hidden width) a resident operand holds

enum Epilogue : int { EP_HIDDEN = 0, EP_HIDDEN_INFER = 1, EP_OUT = 2, EP_DX = 3, EP_DW = 4 };

// Operand kept in shared memory while the other one streams: none (both
// stream; a work unit is one output tile), or B (the whole B, N <= BN, loaded
// once per CTA; a work unit is an M tile: the hidden layers of inference).
// (Keeping an A tile resident across the output layer's N tiles was
// measured: no faster per tile, its work units balance worse.)
enum Resident : int { RES_NONE = 0, RES_B = 1 };

// Words per row of the epilogue staging tile: 36 where a mode writes FP32
// rows, 20 where it writes BF16 rows only (16-byte rows, conflict-free
// quarter warps either way).
template <int MODE>
__host__ __device__ constexpr int stage_pitch() {
  return (MODE == EP_HIDDEN_INFER || MODE == EP_DX) ? 20 : 36;
}
template <int BN, int RES>
__host__ __device__ constexpr int res_box() { return RES == RES_B ? BN * BK * 2 : 0; }
template <int BN, int RES>
__host__ __device__ constexpr int ring_box() { return RES == RES_B ? A_STAGE : A_STAGE + BN * BK * 2; }
template <int BN, int MODE, int RES>
__host__ __device__ constexpr int stages() {
  // as many ring stages (at most 4) as fit beside the resident operand and
  // the staging tiles in 227 KB
  return (232448 - 1024 - 512 - (RES == RES_NONE ? 0 : (K_MAX / BK) * res_box<BN, RES>()) -
          EPI_WARPS * 32 * stage_pitch<MODE>() * 4) / ring_box<BN, RES>() >= 4
             ? 4
             : (232448 - 1024 - 512 - (RES == RES_NONE ? 0 : (K_MAX / BK) * res_box<BN, RES>()) -
                EPI_WARPS * 32 * stage_pitch<MODE>() * 4) / ring_box<BN, RES>();
}

struct GemmArgs {
  int M, N, K;              // C[M, N] = A[M, K] . B[N, K]^T, multiples of 128 / BN / 64
  int mode;
  int m_valid, n_valid;     // rows / columns of the output that are stored
  float* out_f32;           // EP_OUT: y [m_valid, ldo]; EP_DW: gradient [M, ldo]
  int ldo;
  __nv_bfloat16* out_bf16;  // EP_HIDDEN*, EP_DX: [M, ldb]
  int ldb;
  __nv_bfloat16* out_t;     // EP_HIDDEN, EP_DX: transposed [N, ldt]
  int ldt;
  const float* bias;        // EP_HIDDEN*, EP_OUT: [N]
  float* z;                 // EP_HIDDEN: pre-activation written; EP_DX: read; [M, ldz]
  int ldz;
  int* err;
};

// ------------------------------------------------------------ PTX ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred P;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, P;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false (and the error flag raised) after two seconds.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (globaltimer() - t0 > 2000000000ull) {
      atomicOr(err, 1);
      return false;
    }
  }
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(x), "r"(y)
      : "memory");
}
// Shared-memory matrix descriptor of a K-major BF16 tile written by TMA with
// the 128-byte swizzle: rows of 128 bytes, 8-row groups 1024 bytes apart
// (stride byte offset), the leading byte offset unused for this layout,
// descriptor version 1 (bits 46-48), swizzle mode 2 (128 B) in bits 61-63.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16
// A and B (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in
// bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t f16_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tmem_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// SiLU and its derivative through the logistic function written with the
// hardware's approximate hyperbolic tangent, sigma(z) = (1 + tanh(z / 2)) / 2:
// one special-function instruction per element (the epilogue of a hidden
// layer is bound by them; an exponential and a division take two).  Its
// relative error (about 2^-11) is below the BF16 rounding that follows.
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float silu_f(float z) {
  const float h = 0.5f * z;
  return fmaf(h, tanh_approx(h), h);
}
__device__ __forceinline__ float dsilu_f(float z) {
  const float s = fmaf(0.5f, tanh_approx(0.5f * z), 0.5f);
  return s * (1.f + z * (1.f - s));
}

// Row-major store of a warp's 32-row block (thread = row, W 32-bit words
// per row) through the warp's staging tile (P words per row): the block is
// written in the thread-per-row layout and read back so that each lane
// carries VB consecutive bytes of one row and each store instruction writes
// whole rows (full sectors), rows from `row0` of `base` with pitch `pitch`
// bytes.
template <int W, int VB, int P>
__device__ __forceinline__ void store_rows(uint32_t* buf, const uint32_t (&w)[W], int lane, char* base, int row0,
                                           size_t pitch, int rows, int wlim = W) {
  static_assert(W % 4 == 0 && W <= P && P % 4 == 0 && (VB == 16 || VB == 8 || VB == 4), "staged row store shape");
  constexpr int STAGE_PITCH = P;
#pragma unroll
  for (int q = 0; q < W; q += 4)
    *reinterpret_cast<uint4*>(buf + lane * STAGE_PITCH + q) = make_uint4(w[q], w[q + 1], w[q + 2], w[q + 3]);
  __syncwarp();
  constexpr int LPR = W * 4 / VB;    // lanes per row
  constexpr int RPI = 32 / LPR;      // rows per instruction
  const int sub = lane / LPR, q = lane % LPR;
  const int w0 = q * (VB / 4);       // first word of this lane's piece
#pragma unroll 4
  for (int it = 0; it < 32 / RPI; ++it) {
    const int r = it * RPI + sub;
    if (r < rows && w0 < wlim) {
      char* dst = base + (size_t)(row0 + r) * pitch + q * VB;
      const uint32_t* src = buf + r * STAGE_PITCH + w0;
      if (w0 + VB / 4 <= wlim) {
        if (VB == 16) *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(src);
        else if (VB == 8) *reinterpret_cast<uint2*>(dst) = *reinterpret_cast<const uint2*>(src);
        else *reinterpret_cast<uint32_t*>(dst) = *src;
      } else {
        for (int k = 0; w0 + k < wlim; ++k) reinterpret_cast<uint32_t*>(dst)[k] = src[k];
      }
    }
  }
  __syncwarp();
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&p);
}

// Epilogue of a warp's 32 x 32 block: rows row0.. (this thread: row0 +
// lane), columns n..n+31, accumulators v[] in the tcgen05.ld 32x32b layout
// (lane = row, registers = consecutive columns).  The arithmetic runs in that
// layout; row-major outputs leave through store_rows, the transposed copies
// as one BF16 per lane and column (consecutive lanes = consecutive rows).
template <int MODE>
__device__ __forceinline__ void epilogue_chunk(const GemmArgs& a, uint32_t* buf, const float (&v)[32], int row0,
                                               int n, int rows, int lane) {
  const int m = row0 + lane;
  const bool row_ok = lane < rows;
  // bias, four columns at a time (the same address in every lane)
  const float4* bp = reinterpret_cast<const float4*>(a.bias + n);
  if constexpr (MODE == EP_HIDDEN || MODE == EP_HIDDEN_INFER) {
      uint32_t zw[32], hw[16];
#pragma unroll
      for (int q = 0; q < 32; q += 4) {
        const float4 b4 = bp[q / 4];
        zw[q] = __float_as_uint(v[q] + b4.x); zw[q + 1] = __float_as_uint(v[q + 1] + b4.y);
        zw[q + 2] = __float_as_uint(v[q + 2] + b4.z); zw[q + 3] = __float_as_uint(v[q + 3] + b4.w);
      }
      if constexpr (MODE == EP_HIDDEN)
        store_rows<32, 16, stage_pitch<MODE>()>(buf, zw, lane, reinterpret_cast<char*>(a.z + n), row0,
                                                (size_t)a.ldz * 4, rows);
#pragma unroll
      for (int q = 0; q < 16; ++q)
        hw[q] = pack_bf16(silu_f(__uint_as_float(zw[2 * q])), silu_f(__uint_as_float(zw[2 * q + 1])));
      if constexpr (MODE == EP_HIDDEN) {
        if (row_ok) {
          const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(hw);
#pragma unroll
          for (int q = 0; q < 32; ++q) a.out_t[(size_t)(n + q) * a.ldt + m] = h[q];
        }
      }
      store_rows<16, 16, stage_pitch<MODE>()>(buf, hw, lane, reinterpret_cast<char*>(a.out_bf16 + n), row0,
                                              (size_t)a.ldb * 2, rows);
  } else if constexpr (MODE == EP_OUT) {
      uint32_t yw[32];
#pragma unroll
      for (int q = 0; q < 32; q += 4) {
        const float4 b4 = bp[q / 4];
        yw[q] = __float_as_uint(v[q] + b4.x); yw[q + 1] = __float_as_uint(v[q + 1] + b4.y);
        yw[q + 2] = __float_as_uint(v[q + 2] + b4.z); yw[q + 3] = __float_as_uint(v[q + 3] + b4.w);
      }
      // y rows have the caller's pitch: pieces as wide as its alignment allows
      const int wlim = a.n_valid - n < 32 ? a.n_valid - n : 32;
      char* yb = reinterpret_cast<char*>(a.out_f32 + n);
      constexpr int P = stage_pitch<MODE>();
      if ((a.ldo & 3) == 0) store_rows<32, 16, P>(buf, yw, lane, yb, row0, (size_t)a.ldo * 4, rows, wlim);
      else if ((a.ldo & 1) == 0) store_rows<32, 8, P>(buf, yw, lane, yb, row0, (size_t)a.ldo * 4, rows, wlim);
      else store_rows<32, 4, P>(buf, yw, lane, yb, row0, (size_t)a.ldo * 4, rows, wlim);
  } else if constexpr (MODE == EP_DW) {
      uint32_t gw[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) gw[q] = __float_as_uint(v[q]);
      store_rows<32, 16, stage_pitch<MODE>()>(buf, gw, lane, reinterpret_cast<char*>(a.out_f32 + n), row0,
                                              (size_t)a.ldo * 4, rows);
  } else if constexpr (MODE == EP_DX) {
      uint32_t gw[16];
      if (row_ok) {
        const float4* zp = reinterpret_cast<const float4*>(a.z + (size_t)m * a.ldz + n);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const float4 z4 = zp[q];
          gw[2 * q] = pack_bf16(v[4 * q] * dsilu_f(z4.x), v[4 * q + 1] * dsilu_f(z4.y));
          gw[2 * q + 1] = pack_bf16(v[4 * q + 2] * dsilu_f(z4.z), v[4 * q + 3] * dsilu_f(z4.w));
        }
        const __nv_bfloat16* g = reinterpret_cast<const __nv_bfloat16*>(gw);
#pragma unroll
        for (int q = 0; q < 32; ++q) a.out_t[(size_t)(n + q) * a.ldt + m] = g[q];
      } else {
#pragma unroll
        for (int q = 0; q < 16; ++q) gw[q] = 0u;
      }
      store_rows<16, 16, stage_pitch<MODE>()>(buf, gw, lane, reinterpret_cast<char*>(a.out_bf16 + n), row0,
                                              (size_t)a.ldb * 2, rows);
  }
}

// ------------------------------------------------------------ GEMM ----
template <int BN, int MODE, int RES>
__host__ __device__ constexpr size_t gemm_smem_bytes() {
  return 1024 + (RES == RES_NONE ? 0 : (size_t)(K_MAX / BK) * res_box<BN, RES>()) +
         (size_t)stages<BN, MODE, RES>() * ring_box<BN, RES>() + (size_t)EPI_WARPS * 32 * stage_pitch<MODE>() * 4 +
         (2 * stages<BN, MODE, RES>() + 6) * 8 + 16;
}

// Work unit u of the CTA: its M tile and its N tiles [nt0, nt1).
template <int RES>
__device__ __forceinline__ void unit_tiles(int u, int tiles_n, int& mt, int& nt0, int& nt1) {
  if (RES == RES_NONE) { mt = u / tiles_n; nt0 = u % tiles_n; nt1 = nt0 + 1; }
  else { mt = u; nt0 = 0; nt1 = 1; }
}

template <int BN, int MODE, int RES>
__global__ void __launch_bounds__(THREADS, 1)
    k_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, GemmArgs a) {
  constexpr int S = stages<BN, MODE, RES>();
  constexpr int RBOX = res_box<BN, RES>(), SBOX = ring_box<BN, RES>();
  constexpr int P = stage_pitch<MODE>();
  static_assert(S >= 2 && gemm_smem_bytes<BN, MODE, RES>() <= 232448, "shared memory of one CTA");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint8_t* sRes = smem;                                                         // resident operand, K / 64 boxes
  uint8_t* sRing = sRes + (RES == RES_NONE ? 0 : (K_MAX / BK) * RBOX);           // stage ring
  uint32_t* stage_all = reinterpret_cast<uint32_t*>(sRing + S * SBOX);
  uint64_t* bars = reinterpret_cast<uint64_t*>(stage_all + EPI_WARPS * 32 * P);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * S + 6);
  __shared__ volatile int bail;        // a wait of this CTA expired
  __shared__ int issued, res_issued;   // stage loads / resident loads the producer issued
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_n = a.N / BN, tiles_m = (a.M + BM - 1) / BM;
  const int units = RES == RES_NONE ? tiles_m * tiles_n : tiles_m;
  const int nk = a.K / BK;
  const int mlim = (MODE == EP_OUT || MODE == EP_DW) ? a.m_valid : a.M;
  // barriers: full[S], empty[S] (ring), accf[2], acce[2] (accumulators),
  // done, resf (resident operand)
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + S), accf0 = smem_u32(bars + 2 * S),
                 acce0 = smem_u32(bars + 2 * S + 2), done = smem_u32(bars + 2 * S + 4),
                 resf = smem_u32(bars + 2 * S + 5);

  if (threadIdx.x == 0) {
    bail = 0;
    issued = 0;
    res_issued = 0;
    for (int s = 0; s < S; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf0 + 8 * b, 1);
      mbar_init(acce0 + 8 * b, EPI_WARPS);
    }
    mbar_init(done, 1);
    mbar_init(resf, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tmem_fence_before();
  __syncthreads();
  tmem_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // TMA producer
      int g = 0, v = 0;
      for (int u = blockIdx.x; u < units && !bail; u += gridDim.x, ++v) {
        int mt, nt0, nt1;
        unit_tiles<RES>(u, tiles_n, mt, nt0, nt1);
        if (RES == RES_B && v == 0) {
          // the whole B, once per CTA
          mbar_expect_tx(resf, (uint32_t)(nk * RBOX));
          for (int k = 0; k < nk; ++k) tma_load_2d(smem_u32(sRes + k * RBOX), &tb, resf, k * BK, 0);
          res_issued = 1;
        }
        for (int nt = nt0; nt < nt1 && !bail; ++nt) {
          for (int k = 0; k < nk; ++k) {
            const int s = g % S;
            if (g >= S && !mbar_wait(empty0 + 8 * s, ((uint32_t)(g / S) & 1u) ^ 1u, a.err)) { bail = 1; break; }
            mbar_expect_tx(full0 + 8 * s, SBOX);
            uint8_t* st = sRing + s * SBOX;
            tma_load_2d(smem_u32(st), &ta, full0 + 8 * s, k * BK, mt * BM);
            if (RES == RES_NONE) tma_load_2d(smem_u32(st + A_STAGE), &tb, full0 + 8 * s, k * BK, nt * BN);
            ++g;
          }
        }
      }
      issued = g;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer: tile j accumulates into buffer j & 1
      constexpr uint32_t idesc = f16_idesc(BM, BN);
      int g = 0, j = 0, v = 0;
      bool ok = true;
      for (int u = blockIdx.x; u < units && ok && !bail; u += gridDim.x, ++v) {
        int mt, nt0, nt1;
        unit_tiles<RES>(u, tiles_n, mt, nt0, nt1);
        if (RES == RES_B && v == 0) {
          if (!mbar_wait(resf, 0u, a.err)) { ok = false; bail = 1; break; }
          tmem_fence_after();
        }
        for (int nt = nt0; nt < nt1 && ok; ++nt, ++j) {
          const int b = j & 1;
          if (j >= 2 && !mbar_wait(acce0 + 8 * b, ((uint32_t)(j >> 1) & 1u) ^ 1u, a.err)) { ok = false; bail = 1; break; }
          tmem_fence_after();
          const uint32_t acc = tmem + (uint32_t)(b * BN);
          for (int k = 0; k < nk; ++k, ++g) {
            const int s = g % S;
            if (!mbar_wait(full0 + 8 * s, (uint32_t)(g / S) & 1u, a.err)) { ok = false; bail = 1; break; }
            tmem_fence_after();
            const uint32_t st = smem_u32(sRing + s * SBOX);
            const uint32_t a0 = st, b0 = RES == RES_NONE ? st + A_STAGE : smem_u32(sRes + k * RBOX);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk)
              mma_bf16(acc, sw128_desc(a0 + 32 * kk), sw128_desc(b0 + 32 * kk), idesc, (k > 0 || kk > 0) ? 1u : 0u);
            mma_commit(empty0 + 8 * s);
          }
          if (!ok) break;
          mma_commit(accf0 + 8 * b);   // arrives when the tile's MMAs have completed
        }
      }
      mma_commit(done);   // arrives when every MMA issued above has completed
    }
  } else {
    // epilogue: warp w reaches TMEM lanes 32 (w % 4) ..; the warps of a
    // quarter take its 32-column chunks in turn
    const int ew = warp - 2;
    const int quarter = warp & 3;
    constexpr int GROUPS = EPI_WARPS / 4;
    uint32_t* buf = stage_all + ew * 32 * P;
    int j = 0;
    bool ok = true;
    for (int u = blockIdx.x; u < units && ok; u += gridDim.x) {
      int mt, nt0, nt1;
      unit_tiles<RES>(u, tiles_n, mt, nt0, nt1);
      for (int nt = nt0; nt < nt1; ++nt, ++j) {
        const int b = j & 1;
        if (!mbar_wait(accf0 + 8 * b, (uint32_t)(j >> 1) & 1u, a.err)) { ok = false; bail = 1; break; }
        tmem_fence_after();
        const int row0 = mt * BM + quarter * 32, n0 = nt * BN;
        const int rows = mlim - row0 < 32 ? mlim - row0 : 32;
        for (int c0 = (ew >> 2) * 32; c0 < BN; c0 += 32 * GROUPS) {
          float v[32];
          tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * BN + c0), v);
          epilogue_chunk<MODE>(a, buf, v, row0, n0 + c0, rows, lane);
        }
        tmem_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(acce0 + 8 * b);
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // every MMA has completed, and so has every load that was issued (the
    // most recent phase of each stage and of the resident operand; on the
    // normal path all were consumed), before the tensor memory is freed and
    // the CTA exits
    mbar_wait(done, 0, a.err);
    const int g1 = issued;
    for (int g = g1 - S < 0 ? 0 : g1 - S; g < g1; ++g) mbar_wait(full0 + 8 * (g % S), (uint32_t)(g / S) & 1u, a.err);
    if (res_issued > 0) mbar_wait(resf, 0u, a.err);
  }
  tmem_fence_before();
  __syncthreads();
  tmem_fence_after();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN) : "memory");
}

// ------------------------------------------------------- small kernels ----
// x [rows, n_in] (FP32) -> X0 [rpad, kin] BF16 zero-padded, and X0^T [kin, ldt].
__global__ void k_prep_input(const float* x, int64_t rows, int n_in, int64_t rpad, int kin, __nv_bfloat16* x0,
                             __nv_bfloat16* x0t, int ldt) {
  const int64_t total = rpad * kin;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / kin;
    const int c = (int)(e % kin);
    const float v = (r < rows && c < n_in) ? x[r * n_in + c] : 0.f;
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    x0[e] = b;
    if (x0t) x0t[(size_t)c * ldt + r] = b;
  }
}

// Weighted squared error: loss += sum_j w_j (y - t)^2 / B, dY = 2 w_j (y - t) / B
// as BF16 [B, npad] and its transpose [npad, B] (zero in the padded columns).
__global__ void k_loss(const float* y, const float* t, const float* w, int B, int n_out, int npad,
                       __nv_bfloat16* dy, __nv_bfloat16* dyt, double* loss) {
  double acc = 0.0;
  const int64_t total = (int64_t)B * npad;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(e / npad), j = (int)(e % npad);
    float g = 0.f;
    if (j < n_out) {
      const float d = y[(size_t)b * n_out + j] - t[(size_t)b * n_out + j];
      acc += (double)(w[j] * d * d) / B;
      g = 2.f * w[j] * d / (float)B;
    }
    const __nv_bfloat16 gb = __float2bfloat16_rn(g);
    dy[e] = gb;
    dyt[(size_t)j * B + b] = gb;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

// Row sums of a BF16 [n, ld] matrix over its first `cols` columns (the bias
// gradient from the transposed output gradient): one warp per row.
__global__ void k_rowsum(const __nv_bfloat16* a, int n, int ld, int cols, float* out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  float s = 0.f;
  for (int c = lane; c < cols; c += 32) s += __bfloat162float(a[(size_t)warp * ld + c]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[warp] = s;
}

// Adam (Kingma & Ba, 2015) on one FP32 master tensor [n, k] with its
// gradient, moments and the step's bias corrections; refreshes the BF16
// copies [n, k] and [k, n] (wt may be null for a bias).
__global__ void k_adam(float* p, const float* g, float* m1, float* m2, int64_t count, int k, float lr, float b1,
                       float b2, float eps, float c1, float c2, __nv_bfloat16* wb, __nv_bfloat16* wt, int n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x) {
    const float gr = g[e];
    const float a1 = b1 * m1[e] + (1.f - b1) * gr;
    const float a2 = b2 * m2[e] + (1.f - b2) * gr * gr;
    m1[e] = a1;
    m2[e] = a2;
    const float v = p[e] - lr * (a1 / c1) / (sqrtf(a2 / c2) + eps);
    p[e] = v;
    if (wb) {
      const __nv_bfloat16 b = __float2bfloat16_rn(v);
      wb[e] = b;
      if (wt) wt[(size_t)(e % k) * n + e / k] = b;
    }
  }
}

__global__ void k_to_bf16(const float* p, int64_t count, int k, int n, __nv_bfloat16* wb, __nv_bfloat16* wt) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x) {
    const __nv_bfloat16 b = __float2bfloat16_rn(p[e]);
    wb[e] = b;
    wt[(size_t)(e % k) * n + e / k] = b;
  }
}

// ---------------------------------------------------------------- host ----
typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
  static EncodeTiled fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  }
  return fn;
}

// 2-D map of a row-major BF16 matrix [rows, cols] with boxes of 64 columns x box_rows rows, 128-byte swizzle.
bool make_map(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int box_rows) {
  EncodeTiled enc = encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct Layer {
  int n, k;               // padded output and input widths: W [n, k]
  int n_real, k_real;     // logical widths
  float *w, *b, *gw, *gb, *mw, *vw, *mb, *vb;
  __nv_bfloat16 *wb, *wt;  // [n, k], [k, n]
};

}  // namespace

struct mpcmd_mlp {
  mpcmd_mlp_config cfg{};
  int kin = 64, H = 256, L = 4, nout = 0, npad = 0, B = 256;
  int64_t R = 0;           // rows of the activation buffers (>= batch, >= max_rows, multiple of 128)
  std::vector<Layer> layers;
  std::vector<void*> allocs;
  __nv_bfloat16 *x0 = nullptr, *x0t = nullptr;
  std::vector<__nv_bfloat16*> h, ht, dz, dzt;   // [L] activations, transposed, gradients, transposed
  std::vector<float*> z;                        // [L] pre-activations
  __nv_bfloat16 *dy = nullptr, *dyt = nullptr;
  float* yb = nullptr;                          // [B, nout] training output
  double* dloss = nullptr;
  int* derr = nullptr;
  int64_t step = 0;
  int sms = 1;             // SMs of the device (one persistent GEMM CTA each)
  cudaStream_t st = nullptr;

  ~mpcmd_mlp() {
    if (st) cudaStreamDestroy(st);
    for (void* p : allocs) cudaFree(p);
  }
  template <class U>
  int alloc(U*& p, int64_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, sizeof(U) * (size_t)std::max<int64_t>(n, 1)) != cudaSuccess) return MPCMD_ERR_ALLOC;
    allocs.push_back(q);
    cudaMemset(q, 0, sizeof(U) * (size_t)std::max<int64_t>(n, 1));
    p = static_cast<U*>(q);
    return MPCMD_OK;
  }
};

namespace {

int status_of(mpcmd_mlp* m) {
  if (cudaStreamSynchronize(m->st) != cudaSuccess) return MPCMD_ERR_CUDA;
  int e = 0;
  if (cudaMemcpy(&e, m->derr, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return MPCMD_ERR_CUDA;
  return e ? MPCMD_ERR_CUDA : MPCMD_OK;
}

// One persistent CTA per SM (at most one per tile).
template <int BN, int MODE, int RES>
void launch_one(mpcmd_mlp* m, int grid, const CUtensorMap& ta, const CUtensorMap& tb, const GemmArgs& g) {
  k_gemm<BN, MODE, RES><<<grid, THREADS, gemm_smem_bytes<BN, MODE, RES>(), m->st>>>(ta, tb, g);
}

template <int BN>
void launch_bn(mpcmd_mlp* m, int grid, int res, const CUtensorMap& ta, const CUtensorMap& tb, const GemmArgs& g) {
  switch (g.mode) {
    case EP_HIDDEN: launch_one<BN, EP_HIDDEN, RES_NONE>(m, grid, ta, tb, g); break;
    case EP_HIDDEN_INFER:
      if (res == RES_B) launch_one<BN, EP_HIDDEN_INFER, RES_B>(m, grid, ta, tb, g);
      else launch_one<BN, EP_HIDDEN_INFER, RES_NONE>(m, grid, ta, tb, g);
      break;
    case EP_OUT: launch_one<BN, EP_OUT, RES_NONE>(m, grid, ta, tb, g); break;
    case EP_DX: launch_one<BN, EP_DX, RES_NONE>(m, grid, ta, tb, g); break;
    default: launch_one<BN, EP_DW, RES_NONE>(m, grid, ta, tb, g); break;
  }
}

template <int BN, int MODE, int RES>
bool allow_one() {
  return cudaFuncSetAttribute(k_gemm<BN, MODE, RES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)gemm_smem_bytes<BN, MODE, RES>()) == cudaSuccess;
}

template <int BN>
bool allow_smem() {
  return allow_one<BN, EP_HIDDEN, RES_NONE>() && allow_one<BN, EP_HIDDEN_INFER, RES_NONE>() &&
         allow_one<BN, EP_HIDDEN_INFER, RES_B>() && allow_one<BN, EP_OUT, RES_NONE>() &&
         allow_one<BN, EP_DX, RES_NONE>() && allow_one<BN, EP_DW, RES_NONE>();
}

// One persistent CTA per SM (at most one per work unit).  The hidden layers
// of inference keep their weights resident (the whole N fits one tile).
int launch_gemm(mpcmd_mlp* m, const CUtensorMap& ta, const CUtensorMap& tb, const GemmArgs& g, int BN) {
  const int tiles_n = g.N / BN, tiles_m = (g.M + BM - 1) / BM;
  int res = RES_NONE, units = tiles_m * tiles_n;
  if (g.mode == EP_HIDDEN_INFER && tiles_n == 1 && g.K <= K_MAX) {
    res = RES_B;
    units = tiles_m;
  }
  const int grid = units < m->sms ? units : m->sms;
  if (BN == 256) launch_bn<256>(m, grid, res, ta, tb, g);
  else if (BN == 128) launch_bn<128>(m, grid, res, ta, tb, g);
  else launch_bn<64>(m, grid, res, ta, tb, g);
  return cudaPeekAtLastError() == cudaSuccess ? MPCMD_OK : MPCMD_ERR_CUDA;
}

// C[M, N] = A[M, K] . B[N, K]^T on tcgen05; A and B row-major BF16 with
// A_rows x K and B_rows x K allocated (K-major), M, N tile multiples.
int gemm(mpcmd_mlp* m, const void* A, int64_t a_rows, const void* Bm, int64_t b_rows, int M, int N, int K, GemmArgs g,
         int BN) {
  CUtensorMap ta, tb;
  if (!make_map(&ta, A, a_rows, K, BM) || !make_map(&tb, Bm, b_rows, K, BN)) return MPCMD_ERR_CUDA;
  g.M = M; g.N = N; g.K = K; g.err = m->derr;
  return launch_gemm(m, ta, tb, g, BN);
}

int pick_bn(int N) { return N % 256 == 0 ? 256 : (N % 128 == 0 ? 128 : 64); }

// Forward pass of `rows` input rows already in x0 (padded to rp rows); output
// y [rows, nout] FP32 (device).  train: keep pre-activations and the
// transposed activations for the backward pass.
int forward(mpcmd_mlp* m, int64_t rows, int64_t rp, float* y, bool train) {
  const void* in = m->x0;
  int kin = m->kin;
  for (int l = 0; l < m->L; ++l) {
    Layer& ly = m->layers[l];
    GemmArgs g{};
    g.mode = train ? EP_HIDDEN : EP_HIDDEN_INFER;
    g.out_bf16 = m->h[l]; g.ldb = m->H;
    g.out_t = m->ht[l]; g.ldt = (int)m->R;
    g.bias = ly.b;
    g.z = m->z[l]; g.ldz = m->H;
    int r = gemm(m, in, m->R, ly.wb, ly.n, (int)rp, ly.n, kin, g, pick_bn(ly.n));
    if (r) return r;
    in = m->h[l];
    kin = m->H;
  }
  Layer& lo = m->layers[m->L];
  GemmArgs g{};
  g.mode = EP_OUT;
  g.m_valid = (int)rows; g.n_valid = m->nout;
  g.out_f32 = y; g.ldo = m->nout;
  g.bias = lo.b;
  return gemm(m, in, m->R, lo.wb, lo.n, (int)rp, lo.n, m->H, g, pick_bn(lo.n));
}

// Loss and gradients of one batch (inputs x, targets t [B, nout], output
// weights w [nout], device); the gradients land in the layers' gw / gb.
int backward(mpcmd_mlp* m, const float* x, const float* t, const float* w) {
  const int B = m->B;
  k_prep_input<<<256, 256, 0, m->st>>>(x, B, m->cfg.n_in, B, m->kin, m->x0, m->x0t, (int)m->R);
  int r = forward(m, B, B, m->yb, true);
  if (r) return r;
  cudaMemsetAsync(m->dloss, 0, sizeof(double), m->st);
  k_loss<<<256, 256, 0, m->st>>>(m->yb, t, w, B, m->nout, m->npad, m->dy, m->dyt, m->dloss);
  // output layer: dW = dY^T . H_L, db = column sums of dY, dH_L = dY . W
  const __nv_bfloat16* gt = m->dyt;   // [n_l, B] gradient of the current layer's output, transposed
  const __nv_bfloat16* gr = m->dy;    // [B, n_l]
  for (int l = m->L; l >= 0; --l) {
    Layer& ly = m->layers[l];
    const __nv_bfloat16* xin_t = l > 0 ? m->ht[l - 1] : m->x0t;   // layer input, transposed [k, R]
    GemmArgs g{};
    g.mode = EP_DW;
    g.m_valid = ly.n;
    g.out_f32 = ly.gw; g.ldo = ly.k;
    // A = gradient^T [n, B] (pitch B or R), B operand = input^T [k, R] over its first B columns
    const int64_t gt_pitch = (l == m->L) ? B : m->R;
    CUtensorMap ta, tb;
    if (!make_map(&ta, gt, ly.n, gt_pitch, BM) || !make_map(&tb, xin_t, ly.k, m->R, pick_bn(ly.k))) return MPCMD_ERR_CUDA;
    g.M = ly.n; g.N = ly.k; g.K = B; g.err = m->derr;
    r = launch_gemm(m, ta, tb, g, pick_bn(ly.k));
    if (r) return r;
    k_rowsum<<<(ly.n * 32 + 255) / 256, 256, 0, m->st>>>(gt, ly.n, (int)gt_pitch, B, ly.gb);
    if (l == 0) break;
    // input gradient through W and SiLU' of the previous layer's pre-activation
    GemmArgs d{};
    d.mode = EP_DX;
    d.out_bf16 = m->dz[l - 1]; d.ldb = m->H;
    d.out_t = m->dzt[l - 1]; d.ldt = (int)m->R;
    d.z = m->z[l - 1]; d.ldz = m->H;
    r = gemm(m, gr, (l == m->L) ? B : m->R, ly.wt, ly.k, B, ly.k, ly.n, d, pick_bn(ly.k));
    if (r) return r;
    gt = m->dzt[l - 1];
    gr = m->dz[l - 1];
  }
  return cudaPeekAtLastError() == cudaSuccess ? MPCMD_OK : MPCMD_ERR_CUDA;
}

void refresh_bf16(mpcmd_mlp* m) {
  for (Layer& ly : m->layers)
    k_to_bf16<<<256, 256, 0, m->st>>>(ly.w, (int64_t)ly.n * ly.k, ly.k, ly.n, ly.wb, ly.wt);
}

}  // namespace

// ------------------------------------------------------------- C ABI ----
namespace {

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int64_t round_up(int64_t v, int64_t q) { return (v + q - 1) / q * q; }

// Logical (unpadded) parameter layout: per layer W [n_real, k_real] row-major, then b [n_real].
int64_t logical_count(const mpcmd_mlp* m) {
  int64_t c = 0;
  for (const Layer& ly : m->layers) c += (int64_t)ly.n_real * ly.k_real + ly.n_real;
  return c;
}

int copy_params(mpcmd_mlp* m, float* host, bool to_host, bool grads) {
  int64_t off = 0;
  for (Layer& ly : m->layers) {
    std::vector<float> w((size_t)ly.n * ly.k, 0.f), b((size_t)ly.n, 0.f);
    float* dw = grads ? ly.gw : ly.w;
    float* db = grads ? ly.gb : ly.b;
    if (to_host) {
      if (cudaMemcpy(w.data(), dw, 4 * w.size(), cudaMemcpyDeviceToHost) != cudaSuccess) return MPCMD_ERR_CUDA;
      if (cudaMemcpy(b.data(), db, 4 * b.size(), cudaMemcpyDeviceToHost) != cudaSuccess) return MPCMD_ERR_CUDA;
      for (int i = 0; i < ly.n_real; ++i)
        for (int j = 0; j < ly.k_real; ++j) host[off + (int64_t)i * ly.k_real + j] = w[(size_t)i * ly.k + j];
      off += (int64_t)ly.n_real * ly.k_real;
      for (int i = 0; i < ly.n_real; ++i) host[off + i] = b[i];
      off += ly.n_real;
    } else {
      for (int i = 0; i < ly.n_real; ++i)
        for (int j = 0; j < ly.k_real; ++j) w[(size_t)i * ly.k + j] = host[off + (int64_t)i * ly.k_real + j];
      off += (int64_t)ly.n_real * ly.k_real;
      for (int i = 0; i < ly.n_real; ++i) b[i] = host[off + i];
      off += ly.n_real;
      if (cudaMemcpy(dw, w.data(), 4 * w.size(), cudaMemcpyHostToDevice) != cudaSuccess) return MPCMD_ERR_CUDA;
      if (cudaMemcpy(db, b.data(), 4 * b.size(), cudaMemcpyHostToDevice) != cudaSuccess) return MPCMD_ERR_CUDA;
    }
  }
  return MPCMD_OK;
}

}  // namespace

extern "C" {

int mpcmd_mlp_create(const mpcmd_mlp_config* cfg, mpcmd_mlp** out) {
  if (!cfg || !out) return MPCMD_ERR_CONFIG;
  *out = nullptr;
  const mpcmd_mlp_config& c = *cfg;
  if (c.n_in < 1 || c.n_in > 64 || c.n_hidden < 64 || c.n_hidden > 256 || c.n_hidden % 64 || c.n_layers < 1 ||
      c.n_layers > 16 || c.n_out < 1 || c.n_out > (1 << 16) || c.batch < 128 || c.batch % 128 || c.max_rows < 0 ||
      !(c.lr > 0) || !(c.beta1 >= 0 && c.beta1 < 1) || !(c.beta2 >= 0 && c.beta2 < 1) || !(c.eps > 0))
    return MPCMD_ERR_CONFIG;
  if (!encoder()) return MPCMD_ERR_CUDA;
  mpcmd_mlp* m = new mpcmd_mlp();
  m->cfg = c;
  m->kin = 64; m->H = c.n_hidden; m->L = c.n_layers; m->nout = c.n_out; m->B = c.batch;
  m->npad = (int)round_up(c.n_out, 128);
  m->R = round_up(std::max<int64_t>(c.batch, c.max_rows), BM);
  int s = 0;
  if (cudaStreamCreate(&m->st) != cudaSuccess) { delete m; return MPCMD_ERR_CUDA; }
  uint64_t rs = c.seed ? c.seed : 1;
  for (int l = 0; l <= m->L; ++l) {
    Layer ly{};
    const bool out_layer = l == m->L;
    ly.n = out_layer ? m->npad : m->H;
    ly.k = l == 0 ? m->kin : m->H;
    ly.n_real = out_layer ? c.n_out : m->H;
    ly.k_real = l == 0 ? c.n_in : m->H;
    const int64_t nk = (int64_t)ly.n * ly.k;
    s |= m->alloc(ly.w, nk); s |= m->alloc(ly.gw, nk); s |= m->alloc(ly.mw, nk); s |= m->alloc(ly.vw, nk);
    s |= m->alloc(ly.b, ly.n); s |= m->alloc(ly.gb, ly.n); s |= m->alloc(ly.mb, ly.n); s |= m->alloc(ly.vb, ly.n);
    s |= m->alloc(ly.wb, nk); s |= m->alloc(ly.wt, nk);
    if (s) break;
    // Glorot-uniform initial weights on the logical block, zero padding and biases
    std::vector<float> w((size_t)nk, 0.f);
    const double a = std::sqrt(6.0 / (ly.n_real + ly.k_real));
    for (int i = 0; i < ly.n_real; ++i)
      for (int j = 0; j < ly.k_real; ++j)
        w[(size_t)i * ly.k + j] = (float)(a * (2.0 * ((splitmix(rs) >> 11) * (1.0 / 9007199254740992.0)) - 1.0));
    if (cudaMemcpy(ly.w, w.data(), 4 * w.size(), cudaMemcpyHostToDevice) != cudaSuccess) s = MPCMD_ERR_CUDA;
    m->layers.push_back(ly);
  }
  s |= m->alloc(m->x0, m->R * m->kin);
  s |= m->alloc(m->x0t, (int64_t)m->kin * m->R);
  m->h.resize(m->L); m->ht.resize(m->L); m->z.resize(m->L); m->dz.resize(m->L); m->dzt.resize(m->L);
  for (int l = 0; l < m->L && !s; ++l) {
    s |= m->alloc(m->h[l], m->R * m->H);
    s |= m->alloc(m->ht[l], m->R * m->H);
    s |= m->alloc(m->z[l], m->R * m->H);
    s |= m->alloc(m->dz[l], m->R * m->H);
    s |= m->alloc(m->dzt[l], m->R * m->H);
  }
  s |= m->alloc(m->dy, (int64_t)m->B * m->npad);
  s |= m->alloc(m->dyt, (int64_t)m->B * m->npad);
  s |= m->alloc(m->yb, (int64_t)m->B * m->nout);
  s |= m->alloc(m->dloss, 1);
  s |= m->alloc(m->derr, 1);
  if (s) { delete m; return MPCMD_ERR_ALLOC; }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      !allow_smem<256>() || !allow_smem<128>() || !allow_smem<64>()) {
    delete m;
    return MPCMD_ERR_CUDA;
  }
  refresh_bf16(m);
  if (status_of(m)) { delete m; return MPCMD_ERR_CUDA; }
  *out = m;
  return MPCMD_OK;
}

int mpcmd_mlp_destroy(mpcmd_mlp* m) {
  delete m;
  return MPCMD_OK;
}

int mpcmd_mlp_param_count(const mpcmd_mlp* m, int64_t* n) {
  if (!m || !n) return MPCMD_ERR_CONFIG;
  *n = logical_count(m);
  return MPCMD_OK;
}

int mpcmd_mlp_get_params(mpcmd_mlp* m, float* host) {
  if (!m || !host) return MPCMD_ERR_CONFIG;
  if (cudaStreamSynchronize(m->st) != cudaSuccess) return MPCMD_ERR_CUDA;
  return copy_params(m, host, true, false);
}

int mpcmd_mlp_set_params(mpcmd_mlp* m, const float* host) {
  if (!m || !host) return MPCMD_ERR_CONFIG;
  if (cudaStreamSynchronize(m->st) != cudaSuccess) return MPCMD_ERR_CUDA;
  int r = copy_params(m, const_cast<float*>(host), false, false);
  if (r) return r;
  for (Layer& ly : m->layers) {   // a new starting point: fresh moments
    cudaMemsetAsync(ly.mw, 0, 4 * (size_t)ly.n * ly.k, m->st);
    cudaMemsetAsync(ly.vw, 0, 4 * (size_t)ly.n * ly.k, m->st);
    cudaMemsetAsync(ly.mb, 0, 4 * (size_t)ly.n, m->st);
    cudaMemsetAsync(ly.vb, 0, 4 * (size_t)ly.n, m->st);
  }
  m->step = 0;
  refresh_bf16(m);
  return status_of(m);
}

int mpcmd_mlp_forward(mpcmd_mlp* m, const float* x, int64_t rows, float* y) {
  if (!m || !x || !y || rows < 1 || rows > m->R) return MPCMD_ERR_CONFIG;
  const int64_t rp = round_up(rows, BM);
  k_prep_input<<<1024, 256, 0, m->st>>>(x, rows, m->cfg.n_in, rp, m->kin, m->x0, nullptr, (int)m->R);
  int r = forward(m, rows, rp, y, false);
  if (r) return r;
  return status_of(m);
}

int mpcmd_mlp_gradients(mpcmd_mlp* m, const float* x, const float* t, const float* w, float* grads, double* loss) {
  if (!m || !x || !t || !w) return MPCMD_ERR_CONFIG;
  int r = backward(m, x, t, w);
  if (r) return r;
  if ((r = status_of(m))) return r;
  if (loss && cudaMemcpy(loss, m->dloss, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return MPCMD_ERR_CUDA;
  return grads ? copy_params(m, grads, true, true) : MPCMD_OK;
}

int mpcmd_mlp_train_step(mpcmd_mlp* m, const float* x, const float* t, const float* w, double* loss) {
  if (!m || !x || !t || !w) return MPCMD_ERR_CONFIG;
  int r = backward(m, x, t, w);
  if (r) return r;
  m->step += 1;
  const float b1 = (float)m->cfg.beta1, b2 = (float)m->cfg.beta2;
  const float c1 = (float)(1.0 - std::pow(m->cfg.beta1, (double)m->step));
  const float c2 = (float)(1.0 - std::pow(m->cfg.beta2, (double)m->step));
  for (Layer& ly : m->layers) {
    k_adam<<<512, 256, 0, m->st>>>(ly.w, ly.gw, ly.mw, ly.vw, (int64_t)ly.n * ly.k, ly.k, (float)m->cfg.lr, b1, b2,
                                    (float)m->cfg.eps, c1, c2, ly.wb, ly.wt, ly.n);
    k_adam<<<16, 256, 0, m->st>>>(ly.b, ly.gb, ly.mb, ly.vb, ly.n, 1, (float)m->cfg.lr, b1, b2, (float)m->cfg.eps,
                                   c1, c2, nullptr, nullptr, ly.n);
  }
  if (cudaPeekAtLastError() != cudaSuccess) return MPCMD_ERR_CUDA;
  if (loss) {
    if ((r = status_of(m))) return r;
    if (cudaMemcpy(loss, m->dloss, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) return MPCMD_ERR_CUDA;
  }
  return MPCMD_OK;
}

int mpcmd_mlp_synchronize(mpcmd_mlp* m) {
  if (!m) return MPCMD_ERR_CONFIG;
  return status_of(m);
}

}  // extern "C"
