// F_{p^2} arithmetic, p = 2^61 - 1, i^2 = -1, for device and host code.
//
// Replaces virgo::fieldElement (fieldElement.hpp:20-108, fieldElement.cpp).
// Layout: {uint64 re, uint64 im}, 16 bytes, `real` first, exactly the bytes
// the reference memcpy's into Merkle leaves and Fiat-Shamir blocks.
//
// All operations take canonical inputs (each word in [0, p)) and return
// canonical outputs.  For canonical inputs the reference's operators also
// return canonical values equal to the exact field result, so any exact
// evaluation order gives identical bytes; the multiply below uses fewer
// conditional steps than the reference's literal sequence
// (fieldElement.cpp:49-78) but the same value.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define GBZ_HD __host__ __device__ __forceinline__
#else
#define GBZ_HD inline
#endif

namespace gbz {

constexpr uint64_t P = 0x1FFFFFFFFFFFFFFFull;  // 2^61 - 1 (fieldElement.cpp:7)

struct alignas(16) fe {
  uint64_t re, im;
};

GBZ_HD fe fe_make(uint64_t re, uint64_t im) { fe r; r.re = re; r.im = im; return r; }
GBZ_HD fe fe_zero() { return fe_make(0, 0); }
GBZ_HD fe fe_one() { return fe_make(1, 0); }
GBZ_HD bool fe_eq(fe a, fe b) { return a.re == b.re && a.im == b.im; }

// Full 64x64 -> 128 product.
GBZ_HD void mul64wide(uint64_t x, uint64_t y, uint64_t &lo, uint64_t &hi) {
#ifdef __CUDA_ARCH__
  lo = x * y;
  hi = __umul64hi(x, y);
#else
  unsigned __int128 t = (unsigned __int128)x * y;
  lo = (uint64_t)t;
  hi = (uint64_t)(t >> 64);
#endif
}

// x*y mod p without the final reduction: for x, y < 2^62 the value is
// congruent to x*y and below 2^63 + 2^61 (the reference's mymult,
// fieldElement.cpp:341-361, computes the same quantity).
GBZ_HD uint64_t mulp_lazy(uint64_t x, uint64_t y) {
  uint64_t lo, hi;
  mul64wide(x, y, lo, hi);
  return ((hi << 3) | (lo >> 61)) + (lo & P);
}

// Full reduction of any 64-bit value to [0, p).
GBZ_HD uint64_t redp(uint64_t t) {
  t = (t >> 61) + (t & P);  // <= p + 7
  return t >= P ? t - P : t;
}

GBZ_HD uint64_t addp(uint64_t a, uint64_t b) {
  uint64_t s = a + b;
  return s >= P ? s - P : s;
}
GBZ_HD uint64_t subp(uint64_t a, uint64_t b) {
  uint64_t s = a + (P - b);
  return s >= P ? s - P : s;
}

// operator+ (fieldElement.cpp:34-47)
GBZ_HD fe fadd(fe a, fe b) { return fe_make(addp(a.re, b.re), addp(a.im, b.im)); }
// operator- (fieldElement.cpp:80-96)
GBZ_HD fe fsub(fe a, fe b) { return fe_make(subp(a.re, b.re), subp(a.im, b.im)); }
GBZ_HD fe fneg(fe a) { return fsub(fe_zero(), a); }

// Reduction of a value below 2^125 to [0, p): 2^61 = 1 (mod p) folds the
// high part onto the low 61 bits twice, then one conditional subtraction.
GBZ_HD uint64_t red125(unsigned __int128 v) {
  const uint64_t lo = (uint64_t)v, hi = (uint64_t)(v >> 64);
  uint64_t t = ((hi << 3) | (lo >> 61)) + (lo & P);  // < 2^63 + 2^61
  t = (t >> 61) + (t & P);                            // <= p + 4
  return t >= P ? t - P : t;
}

// operator* (fieldElement.cpp:49-78).  The four 122-bit products are
// combined exactly in 128 bits (re = ac - bd + 2p^2, im = ad + bc) and each
// component is reduced once; the reference's Karatsuba form with lazy
// reductions gives the same canonical value, and on the GPU this form
// issues fewer instructions (measured: 331 vs 311 G multiplies/s).
GBZ_HD fe fmul(fe a, fe b) {
  typedef unsigned __int128 u128;
  const u128 ac = (u128)a.re * b.re, bd = (u128)a.im * b.im;
  const u128 ad = (u128)a.re * b.im, bc = (u128)a.im * b.re;
  const u128 bias = (u128)P * P * 2;  // a multiple of p above any bd
  return fe_make(red125(ac + (bias - bd)), red125(ad + bc));
}

GBZ_HD fe fsqr(fe a) { return fmul(a, a); }

// Multiply by a base-field value (img == 0): two products.
GBZ_HD fe fmul_base(fe a, uint64_t c) {
  return fe_make(redp(mulp_lazy(a.re, c)), redp(mulp_lazy(a.im, c)));
}

// fastPow (fieldElement.cpp:323-335) for exponents below 2^64.
GBZ_HD fe fpow(fe x, uint64_t e) {
  fe r = fe_one();
  while (e) {
    if (e & 1) r = fmul(r, x);
    x = fmul(x, x);
    e >>= 1;
  }
  return r;
}

// inv (fieldElement.cpp:207-210): x^(p^2 - 2).  The exponent needs 122
// bits, so it is split as e = hi * 2^64 + lo and x^e = (x^(2^64))^hi * x^lo.
GBZ_HD fe finv(fe x) {
  // p^2 - 2 = 2^122 - 2^62 - 1 ; hi = 2^58 - 1, lo = 2^64 - 2^62 - 1
  const uint64_t lo = 0xBFFFFFFFFFFFFFFFull;
  const uint64_t hi = 0x03FFFFFFFFFFFFFFull;
  fe x64 = x;
  for (int i = 0; i < 64; i++) x64 = fmul(x64, x64);  // x^(2^64)
  return fmul(fpow(x64, hi), fpow(x, lo));
}

// getRootOfUnity (utils.cpp:706-717): generator of order 2^61 squared
// (62 - log_order) times.
GBZ_HD fe root_of_unity(int log_order) {
  fe r = fe_make(2147483648ull, 1033321771269002680ull);
  for (int i = 0; i < 62 - log_order; i++) r = fmul(r, r);
  return r;
}

// quadratic_poly::eval (polynomial.cpp:111-113): ((a x) + b) x + c
GBZ_HD fe quad_eval(fe a, fe b, fe c, fe x) { return fadd(fmul(fadd(fmul(a, x), b), x), c); }

}  // namespace gbz
