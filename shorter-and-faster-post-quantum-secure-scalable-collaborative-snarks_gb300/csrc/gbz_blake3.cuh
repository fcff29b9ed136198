// BLAKE3 of exactly one 64-byte block, for device and host code.
//
// Replaces blake3_hash (Blake3_hash.cpp:5-10), which always hashes 64 bytes
// with the vendored BLAKE3 C library (Blake/blake3.c).  A 64-byte input is a
// single chunk holding a single block, so the hash is one compression with
// the IV as chaining value, counter 0, block length 64 and flags
// CHUNK_START | CHUNK_END | ROOT; the 32-byte output is the first half of
// the state xor the second half.  The message stays in 16 registers and
// the permutation is applied by renaming at compile time.
#pragma once
#include <stdint.h>
#include "gbz_field.cuh"

namespace gbz {

#ifdef __CUDA_ARCH__
GBZ_HD uint32_t b3_rotr(uint32_t x, int c) { return __funnelshift_r(x, x, c); }
#else
GBZ_HD uint32_t b3_rotr(uint32_t x, int c) { return (x >> c) | (x << (32 - c)); }
#endif

#define GBZ_B3_G(a, b, c, d, x, y)      \
  a = a + b + (x);                      \
  d = b3_rotr(d ^ a, 16);               \
  c = c + d;                            \
  b = b3_rotr(b ^ c, 12);               \
  a = a + b + (y);                      \
  d = b3_rotr(d ^ a, 8);                \
  c = c + d;                            \
  b = b3_rotr(b ^ c, 7);

// One round on message words m0..m15 (already permuted for this round).
#define GBZ_B3_ROUND(m0, m1, m2, m3, m4, m5, m6, m7, m8, m9, m10, m11, m12, m13, m14, m15) \
  GBZ_B3_G(v0, v4, v8, v12, m0, m1)                                                        \
  GBZ_B3_G(v1, v5, v9, v13, m2, m3)                                                        \
  GBZ_B3_G(v2, v6, v10, v14, m4, m5)                                                       \
  GBZ_B3_G(v3, v7, v11, v15, m6, m7)                                                       \
  GBZ_B3_G(v0, v5, v10, v15, m8, m9)                                                       \
  GBZ_B3_G(v1, v6, v11, v12, m10, m11)                                                     \
  GBZ_B3_G(v2, v7, v8, v13, m12, m13)                                                      \
  GBZ_B3_G(v3, v4, v9, v14, m14, m15)

// m[16] little-endian message words -> h[8] output words.
GBZ_HD void blake3_block64(const uint32_t m[16], uint32_t h[8]) {
  uint32_t v0 = 0x6A09E667u, v1 = 0xBB67AE85u, v2 = 0x3C6EF372u, v3 = 0xA54FF53Au;
  uint32_t v4 = 0x510E527Fu, v5 = 0x9B05688Cu, v6 = 0x1F83D9ABu, v7 = 0x5BE0CD19u;
  uint32_t v8 = 0x6A09E667u, v9 = 0xBB67AE85u, v10 = 0x3C6EF372u, v11 = 0xA54FF53Au;
  uint32_t v12 = 0, v13 = 0, v14 = 64, v15 = 1u | 2u | 8u;
  const uint32_t M0 = m[0], M1 = m[1], M2 = m[2], M3 = m[3], M4 = m[4], M5 = m[5], M6 = m[6],
                 M7 = m[7], M8 = m[8], M9 = m[9], M10 = m[10], M11 = m[11], M12 = m[12],
                 M13 = m[13], M14 = m[14], M15 = m[15];
  // The message schedule: round r uses sigma^r applied to the indices,
  // sigma = {2,6,3,10,7,0,4,13,1,11,12,5,9,14,15,8}.
  GBZ_B3_ROUND(M0, M1, M2, M3, M4, M5, M6, M7, M8, M9, M10, M11, M12, M13, M14, M15)
  GBZ_B3_ROUND(M2, M6, M3, M10, M7, M0, M4, M13, M1, M11, M12, M5, M9, M14, M15, M8)
  GBZ_B3_ROUND(M3, M4, M10, M12, M13, M2, M7, M14, M6, M5, M9, M0, M11, M15, M8, M1)
  GBZ_B3_ROUND(M10, M7, M12, M9, M14, M3, M13, M15, M4, M0, M11, M2, M5, M8, M1, M6)
  GBZ_B3_ROUND(M12, M13, M9, M11, M15, M10, M14, M8, M7, M2, M5, M3, M0, M1, M6, M4)
  GBZ_B3_ROUND(M9, M14, M11, M5, M8, M12, M15, M1, M13, M3, M0, M10, M2, M6, M4, M7)
  GBZ_B3_ROUND(M11, M15, M5, M0, M1, M9, M8, M6, M14, M10, M2, M12, M3, M4, M7, M13)
  h[0] = v0 ^ v8;
  h[1] = v1 ^ v9;
  h[2] = v2 ^ v10;
  h[3] = v3 ^ v11;
  h[4] = v4 ^ v12;
  h[5] = v5 ^ v13;
  h[6] = v6 ^ v14;
  h[7] = v7 ^ v15;
}

// Message words of four field elements laid out as in memory.
GBZ_HD void fe4_words(fe a, fe b, fe c, fe d, uint32_t m[16]) {
  const fe e[4] = {a, b, c, d};
  for (int i = 0; i < 4; i++) {
    m[4 * i + 0] = (uint32_t)e[i].re;
    m[4 * i + 1] = (uint32_t)(e[i].re >> 32);
    m[4 * i + 2] = (uint32_t)e[i].im;
    m[4 * i + 3] = (uint32_t)(e[i].im >> 32);
  }
}

// hash_F (Fiat_Shamir.cpp:8-27): blake3(x || 0 || y || 0), output bytes
// H[0..7] and H[8..15] folded with weights 2^{7i} into real and img.
GBZ_HD fe hash_F(fe x, fe y) {
  uint32_t m[16], h[8];
  fe4_words(x, fe_zero(), y, fe_zero(), m);
  blake3_block64(m, h);
  uint64_t re = 0, im = 0;
  for (int i = 0; i < 8; i++) {
    uint32_t bre = (h[i >> 2] >> (8 * (i & 3))) & 0xFFu;
    uint32_t bim = (h[2 + (i >> 2)] >> (8 * (i & 3))) & 0xFFu;
    re += (uint64_t)bre << (7 * i);
    im += (uint64_t)bim << (7 * i);
  }
  return fe_make(re, im);
}

// glibc random()/rand(): TYPE_3 additive feedback generator, 31-word table,
// separation 3 (the generator behind F::_random, fieldElement.cpp:119-125,
// and the WHIR query draws, Whir.cpp:262-268).  Seeded like srandom():
// Park-Miller 16807 fill, then 310 outputs discarded.
struct glibc_prng {
  int32_t tbl[31];
  int32_t f, r;
};

GBZ_HD int32_t prng_next(glibc_prng &g) {
  uint32_t v = (uint32_t)g.tbl[g.f] + (uint32_t)g.tbl[g.r];
  g.tbl[g.f] = (int32_t)v;
  int32_t out = (int32_t)(v >> 1);
  if (++g.f >= 31) {
    g.f = 0;
    ++g.r;
  } else if (++g.r >= 31) {
    g.r = 0;
  }
  return out;
}

GBZ_HD void prng_seed(glibc_prng &g, uint32_t seed) {
  if (seed == 0) seed = 1;
  int32_t word = (int32_t)seed;
  g.tbl[0] = word;
  for (int i = 1; i < 31; i++) {
    int32_t hi = word / 127773, lo = word % 127773;
    word = 16807 * lo - 2836 * hi;
    if (word < 0) word += 2147483647;
    g.tbl[i] = word;
  }
  g.f = 3;
  g.r = 0;
  for (int i = 0; i < 310; i++) (void)prng_next(g);
}

// randomNumber (fieldElement.cpp:363-368): 20 decimal digits mod p.
GBZ_HD uint64_t prng_number(glibc_prng &g) {
  uint64_t ret = (uint64_t)(prng_next(g) % 10);
  for (int i = 1; i < 20; i++) {
    ret = ret * 10ull + (uint64_t)(prng_next(g) % 10);
    ret = ret >= P ? ret % P : ret;
  }
  return ret;
}

// F::_random (fieldElement.cpp:119-125)
GBZ_HD fe prng_field(glibc_prng &g) {
  uint64_t re = prng_number(g);
  uint64_t im = prng_number(g);
  return fe_make(re % P, im % P);
}

}  // namespace gbz
