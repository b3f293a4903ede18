/*
 * Random number generators of the oracle (test infrastructure).
 *
 *  - Philox4x32-10, restated from Salmon, Moraes, Dror, Shaw, "Parallel random
 *    numbers: as easy as 1, 2, 3" (SC'11): multipliers 0xD2511F53/0xCD9E8D57,
 *    Weyl key increments 0x9E3779B9/0xBB67AE85, ten rounds.  This is the
 *    "contract" generator shared by the oracle and the GPU engine: every draw
 *    is a pure function of (seed, tag, index, extra, step).
 *  - MT19937 as used by the reference: the 1998 seeding of
 *    collective_code/mtmod.f90:72-85 (sgrnd, LCG 69069) with grnd
 *    (mtmod.f90:88-144, tempered u32 / (2^32-1)), and the 2002 seeding of
 *    selkov_code/mt95.f90:378-404 (init_by_scalar) with genrand_real1
 *    (mt95.f90:828-841: signed int32 * 1/(2^32-1) + 2^31/(2^32-1)).
 */
#include <stdint.h>
#include "oracle.h"

static inline void mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  *lo = (uint32_t)p;
}

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
    mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n1 = lo1;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    uint32_t n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Two words -> double in [0,1) with 53 random bits (exact conversion). */
static inline double u01_from(uint32_t a, uint32_t b) {
  uint64_t m = ((uint64_t)a << 21) | (uint64_t)(b >> 11);
  return (double)m * (1.0 / 9007199254740992.0);
}

double orc_contract_u01(uint64_t seed, uint32_t tag, uint32_t index,
                        uint32_t extra, uint32_t step, int which) {
  uint32_t ctr[4] = {index, extra, step, tag};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t out[4];
  orc_philox4x32_10(ctr, key, out);
  return which ? u01_from(out[2], out[3]) : u01_from(out[0], out[1]);
}

/* ---------------- MT19937 ---------------- */
#define MT_N 624
#define MT_M 397

void orc_mt1998_sgrnd(uint32_t seed, uint32_t* mt) {
  mt[0] = seed;
  for (int i = 1; i < MT_N; ++i) mt[i] = 69069u * mt[i - 1];
}

void orc_mt2002_init(uint32_t seed, uint32_t* mt) {
  mt[0] = seed;
  for (uint32_t i = 1; i < MT_N; ++i)
    mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + i;
}

static void mt_twist(uint32_t* mt) {
  const uint32_t UM = 0x80000000u, LM = 0x7fffffffu, A = 0x9908B0DFu;
  int kk;
  uint32_t y;
  for (kk = 0; kk < MT_N - MT_M; ++kk) {
    y = (mt[kk] & UM) | (mt[kk + 1] & LM);
    mt[kk] = mt[kk + MT_M] ^ (y >> 1) ^ ((y & 1u) ? A : 0u);
  }
  for (; kk < MT_N - 1; ++kk) {
    y = (mt[kk] & UM) | (mt[kk + 1] & LM);
    mt[kk] = mt[kk + (MT_M - MT_N)] ^ (y >> 1) ^ ((y & 1u) ? A : 0u);
  }
  y = (mt[MT_N - 1] & UM) | (mt[0] & LM);
  mt[MT_N - 1] = mt[MT_M - 1] ^ (y >> 1) ^ ((y & 1u) ? A : 0u);
}

static inline uint32_t mt_next(uint32_t* mt, int32_t* mti) {
  if (*mti >= MT_N) { mt_twist(mt); *mti = 0; }
  uint32_t y = mt[(*mti)++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9D2C5680u;
  y ^= (y << 15) & 0xEFC60000u;
  y ^= y >> 18;
  return y;
}

void orc_mt_next_u32(uint32_t* mt, int32_t* mti, uint32_t* out, int64_t n) {
  for (int64_t i = 0; i < n; ++i) out[i] = mt_next(mt, mti);
}

/* mtmod.f90 grnd: unsigned tempered word / (2^32 - 1), in [0,1]. */
double orc_mt_grnd(uint32_t* mt, int32_t* mti) {
  uint32_t y = mt_next(mt, mti);
  return (double)y / (4294967296.0 - 1.0);
}

/* mt95.f90 genrand_real1: signed word * 1/(2^32-1) + 2^31/(2^32-1). */
double orc_mt_real1(uint32_t* mt, int32_t* mti) {
  int32_t a = (int32_t)mt_next(mt, mti);
  const double pi232_1 = 1.0 / (4294967296.0 - 1.0);
  const double p231d232_1 = 2147483648.0 / (4294967296.0 - 1.0);
  return (double)a * pi232_1 + p231d232_1;
}
