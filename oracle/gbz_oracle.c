/*
 * gbz_oracle.c — CPU restatement of the reference prover's hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see gbz_oracle.h).  Each function names the
 * reference file:line it restates.  The arithmetic is exact; where the
 * reference's operation order cannot change a canonical result (all field
 * operations below return the unique representative in [0, p)), loops are
 * reorganised for multi-threading, which is what the CPU baseline needs.
 */
#define _GNU_SOURCE
#include "gbz_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

typedef unsigned __int128 u128;
typedef struct { uint64_t re, im; } fe;

static const uint64_t P = 2305843009213693951ULL; /* fieldElement.cpp:7 */

/* ---------------------------------------------------------------- field */

/* mymult (fieldElement.cpp:341-361): x*y mod p, lazily in [0, 2p). */
static inline uint64_t mymult(uint64_t x, uint64_t y) {
  u128 t = (u128)x * y;
  uint64_t lo = (uint64_t)t, hi = (uint64_t)(t >> 64);
  return ((hi << 3) | (lo >> 61)) + (lo & P);
}
/* myMod (fieldElement.cpp:337-339) */
static inline uint64_t mymod(uint64_t x) { return (x >> 61) + (x & P); }

/* operator+ (fieldElement.cpp:34-47) */
static inline fe f_add(fe a, fe b) {
  fe r;
  r.im = a.im + b.im;
  r.re = a.re + b.re;
  if (P <= r.im) r.im -= P;
  if (P <= r.re) r.re -= P;
  return r;
}
/* operator- (fieldElement.cpp:80-96) */
static inline fe f_sub(fe a, fe b) {
  fe r;
  r.re = a.re + (b.re ^ P);
  r.im = a.im + (b.im ^ P);
  if (r.re >= P) r.re -= P;
  if (r.im >= P) r.im -= P;
  return r;
}
/* operator* (fieldElement.cpp:49-78), step for step. */
static inline fe f_mul(fe a, fe b) {
  fe r;
  uint64_t all = mymult(a.im + a.re, b.im + b.re);
  uint64_t ac = mymult(a.re, b.re), bd = mymult(a.im, b.im);
  uint64_t nac = ac;
  if (bd >= P) bd -= P;
  if (nac >= P) nac -= P;
  nac ^= P;
  bd ^= P;
  uint64_t ti = all + nac + bd;
  ti = mymod(ti);
  if (ti >= P) ti -= P;
  r.im = ti;
  uint64_t tr = ac + bd;
  /* `while (t_real >= mod) t_real -= mod` leaves t_real mod p for any
   * 64-bit t_real; one Mersenne fold plus one subtraction computes the same. */
  tr = mymod(tr);
  if (tr >= P) tr -= P;
  r.re = tr;
  return r;
}
static inline fe f_make(uint64_t re, uint64_t im) { fe r = {re, im}; return r; }
static inline fe f_one(void) { return f_make(1, 0); }
static inline fe f_zero(void) { return f_make(0, 0); }
static inline int f_eq(fe a, fe b) { return a.re == b.re && a.im == b.im; }
/* operator-() (fieldElement.cpp:98-104) = zero() - x */
static inline fe f_neg(fe a) { return f_sub(f_zero(), a); }

/* fastPow (fieldElement.cpp:323-335) */
static fe f_pow(fe x, u128 e) {
  fe ret = f_one(), t = x;
  while (e) {
    if (e & 1) ret = f_mul(ret, t);
    t = f_mul(t, t);
    e >>= 1;
  }
  return ret;
}
/* inv (fieldElement.cpp:207-210): x^(p^2-2) */
static fe f_inv(fe x) {
  u128 p = P;
  return f_pow(x, p * p - 2);
}
/* getRootOfUnity (utils.cpp:706-717 == fieldElement.cpp:238-250) */
static fe f_rou(int n) {
  fe r = f_make(2147483648ULL, 1033321771269002680ULL);
  for (int i = 0; i < 62 - n; i++) r = f_mul(r, r);
  return r;
}
static fe f_small(int64_t x) { /* fieldElement(long long) for small x >= 0 */
  return f_make((uint64_t)x, 0);
}

static inline fe ld(const uint64_t *p, int64_t i) { return f_make(p[2 * i], p[2 * i + 1]); }
static inline void st(uint64_t *p, int64_t i, fe x) { p[2 * i] = x.re; p[2 * i + 1] = x.im; }

void orc_field_ops(int64_t n, const uint64_t *a, const uint64_t *b, uint64_t *add, uint64_t *sub,
                   uint64_t *mul, uint64_t *neg, uint64_t *inv) {
  for (int64_t i = 0; i < n; i++) {
    fe x = ld(a, i), y = ld(b, i);
    if (add) st(add, i, f_add(x, y));
    if (sub) st(sub, i, f_sub(x, y));
    if (mul) st(mul, i, f_mul(x, y));
    if (neg) st(neg, i, f_neg(x));
    if (inv) st(inv, i, f_inv(x));
  }
}

void orc_root_of_unity(int log_order, uint64_t out[2]) {
  fe r = f_rou(log_order);
  out[0] = r.re;
  out[1] = r.im;
}

/* ------------------------------------------------------ glibc random() */
/* glibc's random_r TYPE_3 generator (31-word state, separation 3), seeded
 * by srandom_r's 16807 LCG and 310 discarded outputs.  The reference never
 * calls srand on the prover path, so its generator starts in the state of
 * seed 1 (glibc's static initial table); rand() shares the same state. */
void orc_prng_seed(orc_prng *g, uint32_t seed) {
  if (seed == 0) seed = 1;
  int32_t word = (int32_t)seed;
  g->tbl[0] = word;
  for (int i = 1; i < 31; i++) {
    long hi = word / 127773, lo = word % 127773;
    word = (int32_t)(16807 * lo - 2836 * hi);
    if (word < 0) word += 2147483647;
    g->tbl[i] = word;
  }
  g->f = 3;
  g->r = 0;
  for (int i = 0; i < 310; i++) (void)orc_prng_next(g);
}

int32_t orc_prng_next(orc_prng *g) {
  uint32_t v = (uint32_t)g->tbl[g->f] + (uint32_t)g->tbl[g->r];
  g->tbl[g->f] = (int32_t)v;
  int32_t out = (int32_t)(v >> 1);
  if (++g->f >= 31) {
    g->f = 0;
    ++g->r;
  } else if (++g->r >= 31) {
    g->r = 0;
  }
  return out;
}

/* count random() calls whose outputs are dropped */
void orc_prng_skip(orc_prng *g, uint64_t count) {
  for (uint64_t i = 0; i < count; i++) (void)orc_prng_next(g);
}

/* randomNumber (fieldElement.cpp:363-368) */
static uint64_t prng_number(orc_prng *g) {
  uint64_t ret = (uint64_t)(orc_prng_next(g) % 10);
  for (int i = 1; i < 20; i++) ret = (ret * 10ULL + (uint64_t)(orc_prng_next(g) % 10)) % P;
  return ret;
}
/* _random (fieldElement.cpp:119-125) */
static fe prng_field(orc_prng *g) {
  fe r;
  r.re = prng_number(g) % P;
  r.im = prng_number(g) % P;
  return r;
}
void orc_prng_field(orc_prng *g, uint64_t out[2]) {
  fe r = prng_field(g);
  out[0] = r.re;
  out[1] = r.im;
}

/* -------------------------------------------------------------- BLAKE3 */
/* One BLAKE3 compression of a single 64-byte block, which is the whole
 * hash for a 64-byte input: chaining value = IV, counter 0, block length
 * 64, flags CHUNK_START|CHUNK_END|ROOT.  Algorithm from the BLAKE3
 * specification (vendored as Blake/blake3_portable.c:8-98 and
 * Blake/blake3_impl.h:86-98). */
static const uint32_t B3_IV[8] = {0x6A09E667u, 0xBB67AE85u, 0x3C6EF372u, 0xA54FF53Au,
                                  0x510E527Fu, 0x9B05688Cu, 0x1F83D9ABu, 0x5BE0CD19u};
static const uint8_t B3_PERM[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};

static inline uint32_t rotr32(uint32_t x, int c) { return (x >> c) | (x << (32 - c)); }
static inline void b3g(uint32_t *v, int a, int b, int c, int d, uint32_t x, uint32_t y) {
  v[a] = v[a] + v[b] + x;
  v[d] = rotr32(v[d] ^ v[a], 16);
  v[c] = v[c] + v[d];
  v[b] = rotr32(v[b] ^ v[c], 12);
  v[a] = v[a] + v[b] + y;
  v[d] = rotr32(v[d] ^ v[a], 8);
  v[c] = v[c] + v[d];
  v[b] = rotr32(v[b] ^ v[c], 7);
}

static void blake3_one(const uint8_t in[64], uint8_t out[32]) {
  uint32_t m[16], v[16], t[16];
  for (int i = 0; i < 16; i++)
    m[i] = (uint32_t)in[4 * i] | ((uint32_t)in[4 * i + 1] << 8) | ((uint32_t)in[4 * i + 2] << 16) |
           ((uint32_t)in[4 * i + 3] << 24);
  for (int i = 0; i < 8; i++) v[i] = B3_IV[i];
  v[8] = B3_IV[0]; v[9] = B3_IV[1]; v[10] = B3_IV[2]; v[11] = B3_IV[3];
  v[12] = 0; v[13] = 0; v[14] = 64; v[15] = 1 | 2 | 8;
  for (int r = 0; r < 7; r++) {
    b3g(v, 0, 4, 8, 12, m[0], m[1]);
    b3g(v, 1, 5, 9, 13, m[2], m[3]);
    b3g(v, 2, 6, 10, 14, m[4], m[5]);
    b3g(v, 3, 7, 11, 15, m[6], m[7]);
    b3g(v, 0, 5, 10, 15, m[8], m[9]);
    b3g(v, 1, 6, 11, 12, m[10], m[11]);
    b3g(v, 2, 7, 8, 13, m[12], m[13]);
    b3g(v, 3, 4, 9, 14, m[14], m[15]);
    for (int i = 0; i < 16; i++) t[i] = m[B3_PERM[i]];
    memcpy(m, t, sizeof m);
  }
  for (int i = 0; i < 8; i++) {
    uint32_t o = v[i] ^ v[i + 8];
    out[4 * i] = (uint8_t)o; out[4 * i + 1] = (uint8_t)(o >> 8);
    out[4 * i + 2] = (uint8_t)(o >> 16); out[4 * i + 3] = (uint8_t)(o >> 24);
  }
}

void orc_blake3_64(int64_t count, const uint8_t *in, uint8_t *out) {
  for (int64_t i = 0; i < count; i++) blake3_one(in + 64 * i, out + 32 * i);
}

/* Field element bytes as memcpy'd by the reference: real LE then img LE. */
static inline void fe_bytes(fe x, uint8_t *o) {
  for (int i = 0; i < 8; i++) { o[i] = (uint8_t)(x.re >> (8 * i)); o[8 + i] = (uint8_t)(x.im >> (8 * i)); }
}

/* ------------------------------------------------------- thread helper */
typedef void (*range_fn)(void *ctx, int64_t lo, int64_t hi);
typedef struct { range_fn fn; void *ctx; int64_t lo, hi; } job_t;
static void *job_run(void *p) { job_t *j = (job_t *)p; j->fn(j->ctx, j->lo, j->hi); return NULL; }

static int resolve_threads(int threads) {
  if (threads > 0) return threads;
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  return n > 0 ? (int)n : 1;
}
/* Runs fn over [0, n) split into `threads` contiguous ranges. */
static void parallel_for(int64_t n, int threads, int64_t min_chunk, range_fn fn, void *ctx) {
  threads = resolve_threads(threads);
  if (threads <= 1 || n < 2 * min_chunk) { fn(ctx, 0, n); return; }
  if ((int64_t)threads * min_chunk > n) threads = (int)(n / min_chunk);
  if (threads > 256) threads = 256;
  pthread_t th[256];
  job_t jobs[256];
  for (int t = 0; t < threads; t++) {
    jobs[t].fn = fn; jobs[t].ctx = ctx;
    jobs[t].lo = n * t / threads; jobs[t].hi = n * (t + 1) / threads;
  }
  for (int t = 1; t < threads; t++) pthread_create(&th[t], NULL, job_run, &jobs[t]);
  job_run(&jobs[0]);
  for (int t = 1; t < threads; t++) pthread_join(th[t], NULL);
}

/* ---------------------------------------------------------------- NTT */
/* fft (utils.cpp:904-964): bit-reversal permutation, then radix-2 DIT
 * stages with twiddle w[len/i*k], w[k] = rou^k (rou inverted for the
 * inverse), then scaling by len^{-1} for the inverse. */
typedef struct { fe *a; const fe *w; int64_t len, half, stride; int lghalf; } ntt_stage_ctx;
static void ntt_stage_range(void *p, int64_t lo, int64_t hi) {
  ntt_stage_ctx *c = (ntt_stage_ctx *)p;
  for (int64_t t = lo; t < hi; t++) { /* butterfly index t in [0, len/2) */
    int64_t blk = t >> c->lghalf, k = t & (c->half - 1);
    int64_t j = blk * 2 * c->half;
    fe u = c->a[j + k];
    fe v = f_mul(c->a[j + k + c->half], c->w[c->stride * k]);
    c->a[j + k] = f_add(u, v);
    c->a[j + k + c->half] = f_sub(u, v);
  }
}
typedef struct { fe *w; fe w1; int64_t n; } pow_ctx;
static void pow_range(void *p, int64_t lo, int64_t hi) {
  pow_ctx *c = (pow_ctx *)p;
  fe x = f_pow(c->w1, (u128)lo);
  for (int64_t i = lo; i < hi; i++) { c->w[i] = x; x = f_mul(x, c->w1); }
}
typedef struct { fe *a; fe s; } scale_ctx;
static void scale_range(void *p, int64_t lo, int64_t hi) {
  scale_ctx *c = (scale_ctx *)p;
  for (int64_t i = lo; i < hi; i++) c->a[i] = f_mul(c->a[i], c->s);
}

void orc_fft(uint64_t *data, int logn, int inverse, int threads) {
  int64_t len = (int64_t)1 << logn;
  fe *a = (fe *)data;
  if (len == 1) { /* no butterflies; the inverse still scales by 1^{-1} = 1 */
    if (inverse) a[0] = f_mul(a[0], f_inv(f_one()));
    return;
  }
  for (int64_t i = 1, j = 0; i < len; i++) { /* rev[i] = rev[i>>1]>>1 | (i&1)<<(logn-1) */
    int64_t bit = len >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) { fe t = a[i]; a[i] = a[j]; a[j] = t; }
  }
  fe w1 = f_rou(logn);
  if (inverse) w1 = f_inv(w1);
  fe *w = (fe *)malloc(sizeof(fe) * (size_t)(len / 2));
  pow_ctx pc = {w, w1, len / 2};
  parallel_for(len / 2, threads, 1 << 14, pow_range, &pc);
  int lghalf = 0;
  for (int64_t i = 2; i <= len; i <<= 1, lghalf++) {
    ntt_stage_ctx c = {a, w, len, i >> 1, len / i, lghalf};
    parallel_for(len / 2, threads, 1 << 14, ntt_stage_range, &c);
  }
  free(w);
  if (inverse) {
    scale_ctx sc = {a, f_inv(f_small(len))};
    parallel_for(len, threads, 1 << 14, scale_range, &sc);
  }
}

/* ------------------------------------------------------------- Merkle */
typedef struct { const uint8_t *src; uint8_t *dst; int leaf; } mk_ctx;
static void mk_range(void *p, int64_t lo, int64_t hi) {
  mk_ctx *c = (mk_ctx *)p;
  uint8_t blk[64];
  for (int64_t i = lo; i < hi; i++) {
    if (c->leaf) {
      blake3_one(c->src + 64 * i, c->dst + 32 * i); /* 4 elements = 64 raw bytes */
    } else {
      /* create_tree_blake (merkle_tree.cpp:287-292): both halves of the
       * block are the LEFT child. */
      memcpy(blk, c->src + 32 * (2 * i), 32);
      memcpy(blk + 32, c->src + 32 * (2 * i), 32);
      blake3_one(blk, c->dst + 32 * i);
    }
  }
}

int orc_merkle_commit(const uint64_t *elems, int64_t N, uint8_t *levels_out, int threads) {
  if (N < 4 || (N & (N - 1))) return -1;
  int64_t cnt = N / 4;
  mk_ctx c = {(const uint8_t *)elems, levels_out, 1};
  parallel_for(cnt, threads, 1 << 12, mk_range, &c);
  uint8_t *prev = levels_out;
  while (cnt > 1) {
    uint8_t *next = prev + 32 * cnt;
    cnt /= 2;
    mk_ctx d = {prev, next, 0};
    parallel_for(cnt, threads, 1 << 12, mk_range, &d);
    prev = next;
  }
  return 0;
}

int orc_merkle_open(const uint8_t *levels, int64_t N, int64_t pos, uint8_t *path_out) {
  int64_t cnt = N / 4;
  if (pos < 0 || pos >= cnt) return -1;
  const uint8_t *lv = levels;
  int d = 0;
  while (cnt > 1) {
    int64_t sib = 2 * (pos / 2) + (1 - (pos % 2));
    memcpy(path_out + 32 * d, lv + 32 * sib, 32);
    d++;
    lv += 32 * cnt;
    cnt /= 2;
    pos /= 2;
  }
  return d;
}

/* -------------------------------------------------------- Fiat-Shamir */
/* hash_F (Fiat_Shamir.cpp:8-27): blake3(x || 0 || y || 0), folded to two
 * 56-bit-ish words with weights 2^{7i}. */
static fe hash_F(fe x, fe y) {
  uint8_t data[64], h[32];
  fe z = f_zero();
  fe_bytes(x, data); fe_bytes(z, data + 16); fe_bytes(y, data + 32); fe_bytes(z, data + 48);
  blake3_one(data, h);
  uint64_t re = 0, im = 0;
  for (int i = 0; i < 8; i++) {
    re += (1ULL << (7 * i)) * h[i];
    im += (1ULL << (7 * i)) * h[i + 8];
  }
  return f_make(re, im);
}
void orc_hash_F(const uint64_t x[2], const uint64_t y[2], uint64_t out[2]) {
  fe r = hash_F(f_make(x[0], x[1]), f_make(y[0], y[1]));
  out[0] = r.re; out[1] = r.im;
}
/* hash_to_field (Fiat_Shamir.cpp:29-34) */
static fe fs_absorb(fe *state, const fe *e, int count) {
  for (int i = 0; i < count; i++) *state = hash_F(*state, e[i]);
  return *state;
}
void orc_hash_to_field(uint64_t state[2], const uint64_t *elems, int count, uint64_t out[2]) {
  fe s = f_make(state[0], state[1]);
  fs_absorb(&s, (const fe *)elems, count);
  state[0] = out[0] = s.re;
  state[1] = out[1] = s.im;
}

/* ---------------------------------------------------- beta / evaluate */
/* precompute_beta (utils.cpp:198-243): B[x] = prod_i (bit_i(x) ? r_i : 1-r_i)
 * with bit 0 bound to r[0].  The reference expands r from the last entry;
 * B[2j] = B_j - B_j*r_i, B[2j+1] = B_j*r_i. */
typedef struct { fe *B; const fe *src; fe r; } beta_ctx;
static void beta_range(void *p, int64_t lo, int64_t hi) {
  beta_ctx *c = (beta_ctx *)p;
  for (int64_t j = lo; j < hi; j++) {
    fe t = f_mul(c->r, c->src[j]);
    c->B[2 * j] = f_sub(c->src[j], t);
    c->B[2 * j + 1] = t;
  }
}
void orc_precompute_beta(const uint64_t *r, int nr, uint64_t *Bout, int threads) {
  int64_t n = (int64_t)1 << nr;
  fe *B = (fe *)Bout;
  fe *tmp = (fe *)malloc(sizeof(fe) * (size_t)(n / 2 + 1));
  B[0] = f_one();
  for (int i = 0; i < nr; i++) {
    int64_t cnt = (int64_t)1 << i;
    memcpy(tmp, B, sizeof(fe) * (size_t)cnt);
    beta_ctx c = {B, tmp, ld(r, nr - 1 - i)};
    parallel_for(cnt, threads, 1 << 14, beta_range, &c);
  }
  free(tmp);
}

/* evaluate_vector (utils.cpp:1201-1214): uses the first log2(n) of r. */
void orc_evaluate_vector(const uint64_t *vin, int64_t n, const uint64_t *r, uint64_t out[2]) {
  int lg = 0;
  while (((int64_t)1 << (lg + 1)) <= n) lg++;
  fe *v = (fe *)malloc(sizeof(fe) * (size_t)n);
  memcpy(v, vin, sizeof(fe) * (size_t)n);
  for (int i = 0; i < lg; i++) {
    fe ri = ld(r, i), om = f_sub(f_one(), ri);
    int64_t L = (int64_t)1 << (lg - 1 - i);
    for (int64_t j = 0; j < L; j++) v[j] = f_add(f_mul(om, v[2 * j]), f_mul(ri, v[2 * j + 1]));
  }
  out[0] = v[0].re; out[1] = v[0].im;
  free(v);
}

/* beta_identity (utils.cpp:1337-1343) */
void orc_beta_identity(const uint64_t *r1, const uint64_t *r2, int nr, uint64_t out[2]) {
  fe e = f_one();
  for (int i = 0; i < nr; i++) {
    fe a = ld(r1, i), b = ld(r2, i);
    e = f_mul(e, f_add(f_mul(f_sub(f_one(), a), f_sub(f_one(), b)), f_mul(a, b)));
  }
  out[0] = e.re; out[1] = e.im;
}

/* ----------------------------------------------------------- sumcheck */
/* Round message sum_j (a1 x + b1)(a2 x + b2), a = v[2j+1]-v[2j], b = v[2j]
 * (linear_poly * linear_poly, polynomial.cpp; summed in
 * coSumcheck_MPI.cpp:199 and Whir.cpp:215-221). */
typedef struct { const fe *v1, *v2; fe part[256][3]; int64_t chunk; } sc_ctx;
typedef struct { sc_ctx *c; } sc_arg;
static void sc_range_core(const fe *v1, const fe *v2, int64_t lo, int64_t hi, fe acc[3]) {
  fe A = f_zero(), Bc = f_zero(), C = f_zero();
  for (int64_t j = lo; j < hi; j++) {
    fe a1 = f_sub(v1[2 * j + 1], v1[2 * j]), b1 = v1[2 * j];
    fe a2 = f_sub(v2[2 * j + 1], v2[2 * j]), b2 = v2[2 * j];
    A = f_add(A, f_mul(a1, a2));
    Bc = f_add(Bc, f_add(f_mul(a1, b2), f_mul(b1, a2)));
    C = f_add(C, f_mul(b1, b2));
  }
  acc[0] = A; acc[1] = Bc; acc[2] = C;
}
typedef struct { const fe *v1, *v2; int64_t pairs; int nt; fe part[256][3]; } scp_ctx;
static void scp_range(void *p, int64_t lo, int64_t hi) {
  scp_ctx *c = (scp_ctx *)p;
  for (int64_t t = lo; t < hi; t++) {
    int64_t a = c->pairs * t / c->nt, b = c->pairs * (t + 1) / c->nt;
    sc_range_core(c->v1, c->v2, a, b, c->part[t]);
  }
}
void orc_sumcheck_quadratic(const uint64_t *v1, const uint64_t *v2, int64_t m, uint64_t out[6],
                            int threads) {
  int64_t pairs = m / 2;
  int nt = resolve_threads(threads);
  if (nt > 256) nt = 256;
  if (pairs < ((int64_t)nt << 12)) nt = 1;
  scp_ctx *c = (scp_ctx *)malloc(sizeof(scp_ctx));
  c->v1 = (const fe *)v1; c->v2 = (const fe *)v2; c->pairs = pairs; c->nt = nt;
  parallel_for(nt, nt, 1, scp_range, c);
  fe acc[3] = {f_zero(), f_zero(), f_zero()};
  for (int t = 0; t < nt; t++)
    for (int k = 0; k < 3; k++) acc[k] = f_add(acc[k], c->part[t][k]);
  for (int k = 0; k < 3; k++) { out[2 * k] = acc[k].re; out[2 * k + 1] = acc[k].im; }
  free(c);
}

typedef struct { fe *v, *dst; fe r; } fold_ctx;
static void fold_range(void *p, int64_t lo, int64_t hi) {
  fold_ctx *c = (fold_ctx *)p;
  for (int64_t j = lo; j < hi; j++)
    c->dst[j] = f_add(f_mul(c->r, f_sub(c->v[2 * j + 1], c->v[2 * j])), c->v[2 * j]);
}
/* v[j] = r*(v[2j+1]-v[2j]) + v[2j] (coSumcheck_MPI.cpp:215-218). The
 * in-place reference loop reads index 2j >= j only after writing j, so a
 * copy through a scratch buffer gives the same result in parallel. */
void orc_sumcheck_fold(uint64_t *vin, int64_t m, const uint64_t r[2], int threads) {
  fe *v = (fe *)vin;
  int64_t h = m / 2;
  fe *tmp = (fe *)malloc(sizeof(fe) * (size_t)(h > 0 ? h : 1));
  fold_ctx c = {v, tmp, f_make(r[0], r[1])};
  parallel_for(h, threads, 1 << 14, fold_range, &c);
  memcpy(v, tmp, sizeof(fe) * (size_t)h);
  free(tmp);
}

/* ------------------------------------------------------------ RS folds */
static int ilog2_64(int64_t x) { int l = 0; while (((int64_t)1 << (l + 1)) <= x) l++; return l; }

/* get_RS_multifold_segment_tensor (coPCS_utils.cpp:333-383) */
static fe rs_fold_tensor(const fe *seg, int logk, const fe *r, int64_t n, int64_t idx) {
  int64_t k = (int64_t)1 << logk;
  fe len_inv = f_inv(f_small(k));
  int logn = ilog2_64(n);
  fe om_inv = f_inv(f_rou(logn));
  fe omega = f_pow(om_inv, (u128)(n / k));
  fe inv_om = f_pow(om_inv, (u128)idx);
  fe part[64];
  int64_t seg_n = k;
  fe one = f_one();
  for (int64_t j = 0; j < seg_n / 2; j++) {
    fe s = f_add(seg[j], seg[j + seg_n / 2]), d = f_sub(seg[j], seg[j + seg_n / 2]);
    part[j] = f_add(f_mul(f_sub(one, r[0]), s), f_mul(f_mul(r[0], inv_om), d));
    inv_om = f_mul(inv_om, omega);
  }
  if (logk > 1) {
    fe pw[64];
    pw[0] = one;
    pw[1] = f_mul(om_inv, om_inv);
    for (int i = 2; i < logk; i++) pw[i] = f_mul(pw[i - 1], pw[i - 1]);
    for (int i = 1; i < logk; i++) pw[i] = f_pow(pw[i], (u128)(n / seg_n));
    for (int i = 1; i < logk; i++) {
      seg_n /= 2;
      fe o = f_inv(f_rou(ilog2_64(n >> i)));
      fe po = f_pow(o, (u128)idx);
      for (int64_t j = 0; j < seg_n / 2; j++) {
        fe s = f_add(part[j], part[j + seg_n / 2]), d = f_sub(part[j], part[j + seg_n / 2]);
        part[j] = f_add(f_mul(f_sub(one, r[i]), s), f_mul(r[i], f_mul(po, d)));
        po = f_mul(po, pw[i]);
      }
    }
  }
  return f_mul(len_inv, part[0]);
}
void orc_rs_fold_tensor(const uint64_t *segment, int logk, const uint64_t *r, int64_t n, int64_t idx,
                        uint64_t out[2]) {
  fe y = rs_fold_tensor((const fe *)segment, logk, (const fe *)r, n, idx);
  out[0] = y.re; out[1] = y.im;
}

/* RS_multifold5 (coPCS_utils.cpp:386-437): each output i gathers the d
 * entries cw[i + t*n/d] through log2(d) inverse-twiddled butterfly levels,
 * then y_i = d^{-1} * sum_j a_j * partial_i[j]. */
typedef struct { const fe *cw; int64_t n; const fe *a; int logd; fe *out; fe len_inv, om_inv; const fe *pw; } mf5_ctx;
static void mf5_range(void *p, int64_t lo, int64_t hi) {
  mf5_ctx *c = (mf5_ctx *)p;
  int64_t d = (int64_t)1 << c->logd, n = c->n;
  fe buf[2][64];
  for (int64_t i = lo; i < hi; i++) {
    /* level 0 pairs (j, j + n/2) for the d/2 indices j = i + t*n/d */
    fe cur[64];
    int64_t cnt = d / 2;
    for (int64_t t = 0; t < cnt; t++) {
      int64_t j = i + t * (n / d);
      fe s = f_add(c->cw[j], c->cw[j + n / 2]);
      fe df = f_mul(f_pow(c->om_inv, (u128)j), f_sub(c->cw[j], c->cw[j + n / 2]));
      buf[0][2 * t] = s; buf[0][2 * t + 1] = df; /* partial[j] = {s, df} */
    }
    /* partial index for position j (t-th) is a vector of length 2; now
     * merge levels: at level lv the vector for j (j < n/2^{lv+1}) takes
     * partner j + n/2^{lv+1}. */
    int64_t width = 2, groups = cnt; /* groups of `width` entries */
    fe *src = buf[0], *dst = buf[1];
    for (int lv = 1; lv < c->logd; lv++) {
      int64_t ng = groups / 2;
      int64_t nn = n >> lv; /* n after halving */
      for (int64_t g = 0; g < ng; g++) {
        int64_t j = i + g * (n / d); /* index of the kept vector */
        int64_t e = j; /* pow_omega exponent = loop index j in the reference */
        fe po = f_pow(c->pw[lv], (u128)e);
        for (int64_t k = 0; k < width; k++) {
          fe x = src[g * width + k], y = src[(g + ng) * width + k];
          dst[g * 2 * width + k] = f_add(x, y);
          dst[g * 2 * width + k + width] = f_mul(po, f_sub(x, y));
        }
        (void)nn;
      }
      width *= 2;
      groups = ng;
      fe *t = src; src = dst; dst = t;
    }
    fe acc = f_zero();
    for (int64_t k = 0; k < d; k++) acc = f_add(acc, f_mul(c->a[k], src[k]));
    cur[0] = f_mul(acc, c->len_inv);
    c->out[i] = cur[0];
  }
}
void orc_rs_multifold5(const uint64_t *codeword, int64_t n, const uint64_t *a, int logd, uint64_t *out,
                       int threads) {
  int64_t d = (int64_t)1 << logd;
  fe om_inv = f_inv(f_rou(ilog2_64(n)));
  fe pw[64];
  pw[0] = f_one();
  if (logd > 1) pw[1] = f_mul(om_inv, om_inv);
  for (int i = 2; i < logd; i++) pw[i] = f_mul(pw[i - 1], pw[i - 1]);
  mf5_ctx c = {(const fe *)codeword, n, (const fe *)a, logd, (fe *)out, f_inv(f_small(d)), om_inv, pw};
  parallel_for(n / d, threads, 1 << 10, mf5_range, &c);
}

/* ------------------------------------------------------- update_betas */
typedef struct { fe *b; const fe *w, *c; int l; } ub_ctx;
static void ub_range(void *p, int64_t lo, int64_t hi) {
  ub_ctx *c = (ub_ctx *)p;
  for (int i = 0; i < c->l; i++) {
    fe x = f_mul(c->c[i], f_pow(c->w[i], (u128)lo));
    for (int64_t j = lo; j < hi; j++) {
      c->b[j] = f_add(c->b[j], x);
      x = f_mul(x, c->w[i]);
    }
  }
}
/* update_betas (Whir.cpp:325-342) with compute_powers_vector (:316-323):
 * b[j] += c_i * (omega_N^{q_i})^j; the sum over i is exact, so grouping
 * the additions per j-range instead of per query gives the same values. */
void orc_update_betas(uint64_t *b, int64_t nb, const int32_t *queries, int l, int64_t N, const uint64_t r[2],
                      uint64_t *challenges_out, int threads) {
  fe rr = f_make(r[0], r[1]);
  fe *c = (fe *)malloc(sizeof(fe) * (size_t)(l > 0 ? l : 1));
  fe *w = (fe *)malloc(sizeof(fe) * (size_t)(l > 0 ? l : 1));
  fe om = f_rou(ilog2_64(N));
  for (int i = 0; i < l; i++) {
    c[i] = i == 0 ? rr : f_mul(c[i - 1], rr);
    w[i] = f_pow(om, (u128)(uint32_t)queries[i]);
    if (challenges_out) st(challenges_out, i, c[i]);
  }
  ub_ctx u = {(fe *)b, w, c, l};
  parallel_for(nb, threads, 1 << 10, ub_range, &u);
  free(c);
  free(w);
}

int orc_whir_queries(int rate) {
  return (int)(-100.0 / log2(sqrt(1.0 / (double)rate)));
}

/* --------------------------------------------------------- transcript */
enum {
  T_COMMIT_ROOT = 1, T_EVAL_POINT = 2, T_CLAIM = 3, T_SC_POLY = 4, T_SC_CHALLENGE = 5,
  T_SC_FINAL = 6, T_WHIR_POLY = 7, T_WHIR_CHALLENGE = 8, T_WHIR_ROOT = 9,
  T_WHIR_QUERIES = 10, T_WHIR_REPLIES = 11, T_WHIR_ANSWERS = 12, T_WHIR_PATHS = 13,
  T_WHIR_COMBINE = 14, T_WHIR_K = 15, T_FINAL_POLY = 16, T_FINAL_POINT = 17,
  T_FINAL_EVAL = 18
};

typedef struct { uint8_t *p; int64_t len, cap; int bad; } tw_t;
static uint8_t *tw_rec(tw_t *t, uint32_t tag, uint32_t count, size_t unit) {
  int64_t need = 8 + (int64_t)unit * count;
  if (t->bad || t->len + need > t->cap) { t->bad = 1; t->len += need; return NULL; }
  uint8_t *o = t->p + t->len;
  memcpy(o, &tag, 4);
  memcpy(o + 4, &count, 4);
  t->len += need;
  return o + 8;
}
static void tw_fe(tw_t *t, uint32_t tag, const fe *v, uint32_t count) {
  uint8_t *o = tw_rec(t, tag, count, 16);
  if (o) for (uint32_t i = 0; i < count; i++) fe_bytes(v[i], o + 16 * i);
}
static void tw_raw(tw_t *t, uint32_t tag, const void *v, uint32_t count, size_t unit) {
  uint8_t *o = tw_rec(t, tag, count, unit);
  if (o) memcpy(o, v, unit * count);
}

static fe quad_eval(const fe h[3], fe x) { /* ((a x) + b) x + c */
  return f_add(f_mul(f_add(f_mul(h[0], x), h[1]), x), h[2]);
}

/* Whir_Commit_initial (Whir.cpp:158-190): codeword = pfft(arr padded to
 * rate*|arr|), tree = MT_commit_Blake(codeword). */
static void whir_commit(const fe *arr, int64_t m, int rate, fe **cw_out, uint8_t **tree_out, int threads) {
  int64_t L = m * rate;
  fe *cw = (fe *)calloc((size_t)L, sizeof(fe));
  memcpy(cw, arr, sizeof(fe) * (size_t)m);
  orc_fft((uint64_t *)cw, ilog2_64(L), 0, threads);
  uint8_t *tree = (uint8_t *)malloc((size_t)32 * (size_t)(L / 2 > 1 ? L / 2 : 1));
  orc_merkle_commit((const uint64_t *)cw, L, tree, threads);
  *cw_out = cw;
  *tree_out = tree;
}
static const uint8_t *tree_root(const uint8_t *tree, int64_t L) {
  return tree + 32 * (L / 2 - 2); /* (L/2 - 1) hashes, root last */
}

int64_t orc_transcript_bytes(int logn, int rate) {
  /* Exact length of orc_prove's record sequence. */
  int64_t n = (int64_t)1 << logn;
  int64_t bytes = 0;
  bytes += 8 + 32 + 8 + 16 * logn + 8 + 16;           /* root, point, claim */
  bytes += (int64_t)logn * (8 + 48 + 8 + 16) + 8 + 32; /* sumcheck */
  int64_t m = n, L = n * rate;
  int cur = rate;
  for (;;) {
    bytes += 2 * (8 + 48 + 8 + 16) + 8 + 32;
    int l = orc_whir_queries(cur);
    int depth = ilog2_64(L / 4);
    bytes += 8 + 4 * l + 8 + 64 * l + 8 + 16 * l + 8 + 32 * (int64_t)l * depth + 8 + 16 * l + 8 + 16;
    m /= 4;
    L = m * 2 * cur;
    cur *= 2;
    if (m <= 4) break;
  }
  bytes += 8 + 16 * m + 8 + 16 * (int64_t)ilog2_64(m) + 8 + 16;
  return bytes;
}

void orc_witness(uint64_t seed, int64_t n, uint64_t *out) {
  uint64_t s = seed;
  for (int64_t i = 0; i < n; i++) {
    uint64_t v;
    do {
      uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
      z ^= z >> 31;
      v = z >> 3;
    } while (v == P);
    out[2 * i] = v;
    out[2 * i + 1] = 0;
  }
}

/* The plain single-party prover (restating oracle/ref/ref_driver.cpp
 * cmd_prove, which calls the reference's Whir_Commit_initial, hash_to_field,
 * precompute_beta, the _quadratic_cosumcheck round body, whir_sumcheck_step1/2,
 * whir_query, open_tree_blake, update_betas, evaluate_vector). */
int64_t orc_prove(const uint64_t *witness, int logn, int rate, uint32_t prng_seed, uint8_t *transcript,
                  int64_t cap, int threads) {
  const int whir_k = 4, logk = 2;
  if (logn < 3 || logn > 30 || rate < 2 || (rate & (rate - 1))) return -1;
  int64_t n = (int64_t)1 << logn;
  tw_t tw = {transcript, 0, cap, 0};
  orc_prng g;
  orc_prng_seed(&g, prng_seed);
  fe fs = f_zero();
  const fe *w = (const fe *)witness;

  /* 1. commitment */
  fe *cw;
  uint8_t *tree;
  whir_commit(w, n, rate, &cw, &tree, threads);
  int64_t L = n * rate;
  tw_raw(&tw, T_COMMIT_ROOT, tree_root(tree, L), 1, 32);

  /* 2. evaluation point z_i = hash_to_field({0}) (main.cpp:83-85) */
  fe *z = (fe *)malloc(sizeof(fe) * (size_t)logn);
  fe zero = f_zero();
  for (int i = 0; i < logn; i++) z[i] = fs_absorb(&fs, &zero, 1);
  tw_fe(&tw, T_EVAL_POINT, z, (uint32_t)logn);
  fe *v1 = (fe *)malloc(sizeof(fe) * (size_t)n), *v2 = (fe *)malloc(sizeof(fe) * (size_t)n);
  orc_precompute_beta((const uint64_t *)z, logn, (uint64_t *)v2, threads);
  memcpy(v1, w, sizeof(fe) * (size_t)n);

  /* 3. sumcheck of sum_x w(x) eq(z, x) with Fiat-Shamir challenges */
  fe *chal = (fe *)malloc(sizeof(fe) * (size_t)logn);
  fe y = f_zero();
  int64_t m = n;
  for (int i = 0; i < logn; i++) {
    uint64_t H6[6];
    orc_sumcheck_quadratic((const uint64_t *)v1, (const uint64_t *)v2, m, H6, threads);
    fe H[3] = {f_make(H6[0], H6[1]), f_make(H6[2], H6[3]), f_make(H6[4], H6[5])};
    if (i == 0) {
      y = f_add(quad_eval(H, f_zero()), quad_eval(H, f_one()));
      tw_fe(&tw, T_CLAIM, &y, 1);
    }
    tw_fe(&tw, T_SC_POLY, H, 3);
    chal[i] = fs_absorb(&fs, H, 3);
    tw_fe(&tw, T_SC_CHALLENGE, &chal[i], 1);
    y = quad_eval(H, chal[i]);
    uint64_t c2[2] = {chal[i].re, chal[i].im};
    orc_sumcheck_fold((uint64_t *)v1, m, c2, threads);
    orc_sumcheck_fold((uint64_t *)v2, m, c2, threads);
    m /= 2;
  }
  fe fin[2] = {v1[0], v2[0]};
  tw_fe(&tw, T_SC_FINAL, fin, 2);

  /* 4. WHIR open of (v1[0], chal) with whir_k = 4 (Whir_Open, Whir.cpp:388-467) */
  fe K = v1[0];
  fe *b = v2; /* reuse: b = precompute_beta(chal) */
  orc_precompute_beta((const uint64_t *)chal, logn, (uint64_t *)b, threads);
  fe *arr = v1;
  memcpy(arr, w, sizeof(fe) * (size_t)n);
  m = n;
  int cur = rate;
  for (;;) {
    fe r[2];
    for (int i = 0; i < logk; i++) {
      uint64_t H6[6];
      orc_sumcheck_quadratic((const uint64_t *)arr, (const uint64_t *)b, m, H6, threads);
      fe h[3] = {f_make(H6[0], H6[1]), f_make(H6[2], H6[3]), f_make(H6[4], H6[5])};
      tw_fe(&tw, T_WHIR_POLY, h, 3);
      r[i] = prng_field(&g);
      tw_fe(&tw, T_WHIR_CHALLENGE, &r[i], 1);
      K = quad_eval(h, r[i]);
      uint64_t c2[2] = {r[i].re, r[i].im};
      orc_sumcheck_fold((uint64_t *)arr, m, c2, threads);
      orc_sumcheck_fold((uint64_t *)b, m, c2, threads);
      m /= 2;
    }
    fe *ncw;
    uint8_t *ntree;
    whir_commit(arr, m, 2 * cur, &ncw, &ntree, threads);
    int64_t NL = m * 2 * cur;
    tw_raw(&tw, T_WHIR_ROOT, tree_root(ntree, NL), 1, 32);

    /* whir_query (Whir.cpp:251-314) on the previous codeword */
    int l = orc_whir_queries(cur);
    int32_t *q = (int32_t *)malloc(sizeof(int32_t) * (size_t)l);
    for (int i = 0; i < l; i++) q[i] = orc_prng_next(&g) % (int32_t)(L / 4); /* whir_k <= 4 */
    tw_raw(&tw, T_WHIR_QUERIES, q, (uint32_t)l, 4);
    fe *rep = (fe *)malloc(sizeof(fe) * (size_t)l * whir_k);
    fe *ans = (fe *)malloc(sizeof(fe) * (size_t)l);
    for (int i = 0; i < l; i++) {
      for (int j = 0; j < whir_k; j++) rep[i * whir_k + j] = cw[q[i] + j * (L / whir_k)];
      ans[i] = rs_fold_tensor(rep + i * whir_k, logk, r, L, q[i]);
    }
    tw_fe(&tw, T_WHIR_REPLIES, rep, (uint32_t)(l * whir_k));
    tw_fe(&tw, T_WHIR_ANSWERS, ans, (uint32_t)l);
    int depth = ilog2_64(L / 4);
    uint8_t *paths = (uint8_t *)malloc((size_t)32 * (size_t)l * (size_t)(depth > 0 ? depth : 1));
    for (int i = 0; i < l; i++) orc_merkle_open(tree, L, q[i], paths + (size_t)32 * depth * i);
    tw_raw(&tw, T_WHIR_PATHS, paths, (uint32_t)(l * depth), 32);
    free(paths);
    free(rep);

    /* queries scaled to the new codeword (Whir.cpp:371-372), update_betas */
    for (int i = 0; i < l; i++) q[i] = q[i] * (int32_t)(whir_k * NL / L);
    free(cw);
    free(tree);
    cw = ncw;
    tree = ntree;
    L = NL;
    fe rb = prng_field(&g);
    fe *ch = (fe *)malloc(sizeof(fe) * (size_t)l);
    uint64_t rb2[2] = {rb.re, rb.im};
    orc_update_betas((uint64_t *)b, m, q, l, L, rb2, (uint64_t *)ch, threads);
    tw_fe(&tw, T_WHIR_COMBINE, ch, (uint32_t)l);
    for (int i = 0; i < l; i++) K = f_add(K, f_mul(ch[i], ans[i]));
    tw_fe(&tw, T_WHIR_K, &K, 1);
    free(ch);
    free(ans);
    free(q);
    cur *= 2;
    if (m <= whir_k) break;
  }
  tw_fe(&tw, T_FINAL_POLY, arr, (uint32_t)m);
  int lgm = ilog2_64(m);
  fe rf[8];
  for (int i = 0; i < lgm; i++) rf[i] = prng_field(&g);
  tw_fe(&tw, T_FINAL_POINT, rf, (uint32_t)lgm);
  uint64_t ev[2];
  orc_evaluate_vector((const uint64_t *)b, m, (const uint64_t *)rf, ev);
  fe e = f_make(ev[0], ev[1]);
  tw_fe(&tw, T_FINAL_EVAL, &e, 1);

  free(cw);
  free(tree);
  free(z);
  free(chal);
  free(v1);
  free(v2);
  return tw.bad ? -1 : tw.len;
}

/* ============================================================ coPCS side */

void orc_lagrange_coeff(const uint64_t r[2], int logd, uint64_t *out) {
  int64_t d = (int64_t)1 << logd;
  fe rr = f_make(r[0], r[1]), x = f_one();
  for (int64_t i = 0; i < d; i++) { st(out, i, x); x = f_mul(x, rr); }
  orc_fft(out, logd, 1, 1);
}

void orc_encode_rows(const uint64_t *rows, int nrows, int logrow, int rate, int log_rate_offset, uint64_t *out,
                     int threads) {
  int64_t n = (int64_t)1 << logrow, L = n * rate;
  fe w = f_inv(f_rou(1 + log_rate_offset + logrow));
  for (int i = 0; i < nrows; i++) {
    uint64_t *o = out + 2 * L * i;
    memset(o, 0, sizeof(uint64_t) * 2 * L);
    memcpy(o, rows + 2 * n * i, sizeof(uint64_t) * 2 * n);
    orc_fft(o, logrow, 1, threads);
    fe mul = f_one();
    for (int64_t j = 0; j < n; j++) { st(o, j, f_mul(mul, ld(o, j))); mul = f_mul(mul, w); }
    orc_fft(o, ilog2_64(L), 0, threads);
  }
}

static void hash_self(const uint8_t in[32], uint8_t out[32]) {  /* blake3(x || x) */
  uint8_t blk[64];
  memcpy(blk, in, 32);
  memcpy(blk + 32, in, 32);
  blake3_one(blk, out);
}

void orc_column_merkle(const uint64_t *rows, int nrows, int logL, int N, uint8_t *levels, uint8_t root_out[32]) {
  int64_t L = (int64_t)1 << logL;
  /* column j: MT_commit_Blake over the 32-element batch vector; its root
   * only depends on the first leaf (rows 0..3) because inner nodes hash
   * their left child twice, but the full tree is built here as in the
   * reference. */
  for (int64_t j = 0; j < L; j++) {
    uint64_t col[64];
    memset(col, 0, sizeof col);
    for (int k = 0; k < nrows && k < 32; k++) { col[2 * k] = rows[2 * (L * k + j)]; col[2 * k + 1] = rows[2 * (L * k + j) + 1]; }
    uint8_t lv[15 * 32];
    orc_merkle_commit(col, 32, lv, 1);
    memcpy(levels + 32 * j, lv + 32 * 14, 32);
  }
  /* create_tree_blake over the column roots */
  uint8_t *prev = levels;
  int64_t cnt = L;
  while (cnt > 1) {
    uint8_t *next = prev + 32 * cnt;
    cnt /= 2;
    for (int64_t i = 0; i < cnt; i++) hash_self(prev + 32 * (2 * i), next + 32 * i);
    prev = next;
  }
  /* leader: tree over {root, 0, ..., 0} of N parties; its root is the left chain */
  uint8_t cur[32];
  memcpy(cur, prev, 32);
  for (int n = N; n > 1; n /= 2) { uint8_t t[32]; hash_self(cur, t); memcpy(cur, t, 32); }
  memcpy(root_out, cur, 32);
}

/* compute_secret_shares per group (MPI_utils.cpp:2747-2762): inverse
 * transform of the _k group values, zero-pad to 2N, forward transform, party
 * j takes entry 2j+1.  The map is linear, so it is built once (the images of
 * the unit vectors through the same transforms) and applied to every group;
 * the groups' random slots are drawn first, in the reference's order. */
typedef struct { const uint64_t *v, *fill; const fe *mu; int64_t groups; int N, k, kk; uint64_t *shares; } shr_ctx;
static void shares_range(void *p, int64_t lo, int64_t hi) {
  shr_ctx *c = (shr_ctx *)p;
  fe buf[32];
  for (int64_t i = lo; i < hi; i++) {
    for (int t = 0; t < c->k; t++) buf[t] = ld(c->v, i * c->k + t);
    for (int t = c->k; t < c->kk; t++) buf[t] = c->fill ? ld(c->fill, i * (c->kk - c->k) + (t - c->k)) : f_zero();
    for (int j = 0; j < c->N; j++) {
      fe acc = f_zero();
      for (int t = 0; t < c->kk; t++) acc = f_add(acc, f_mul(c->mu[j * c->kk + t], buf[t]));
      st(c->shares, j * c->groups + i, acc);
    }
  }
}

void orc_secret_shares_g(const uint64_t *v, int64_t M, int N, int privacy, orc_prng *g, uint64_t *shares) {
  int k = N / 4, kk = N / 2;
  int64_t groups = M / k;
  int lk = ilog2_64(kk), l2n = ilog2_64(2 * N);
  fe *mu = (fe *)malloc(sizeof(fe) * (size_t)N * kk);
  uint64_t buff[2 * 256];
  for (int t = 0; t < kk; t++) {
    memset(buff, 0, sizeof(uint64_t) * 2 * 2 * N);
    buff[2 * t] = 1;
    orc_fft(buff, lk, 1, 1);
    orc_fft(buff, l2n, 0, 1);
    for (int j = 0; j < N; j++) mu[j * kk + t] = ld(buff, 2 * j + 1);
  }
  uint64_t *fill = NULL;
  if (privacy && kk > k) {
    fill = (uint64_t *)malloc(sizeof(uint64_t) * 2 * (size_t)(groups * (kk - k)));
    for (int64_t i = 0; i < groups * (kk - k); i++) { fill[2 * i] = (uint64_t)orc_prng_next(g); fill[2 * i + 1] = 0; }
  }
  shr_ctx c = {v, fill, mu, groups, N, k, kk, shares};
  parallel_for(groups, 0, 1 << 12, shares_range, &c);
  free(fill);
  free(mu);
}

void orc_secret_shares(const uint64_t *v, int64_t M, int N, int privacy, uint32_t prng_seed, uint64_t *shares) {
  orc_prng g;
  orc_prng_seed(&g, prng_seed);
  orc_secret_shares_g(v, M, N, privacy, &g, shares);
}

void orc_generate_randomness(orc_prng *g, int64_t n, uint64_t *out) {
  uint64_t c = 0;
  for (int64_t i = 0; i < n; i++) {
    if (i % 100 == 0) c = (uint64_t)orc_prng_next(g); /* c = random() */
    out[2 * i] = c + (uint64_t)orc_prng_next(g);       /* c + F(rand()): both below 2^31 */
    out[2 * i + 1] = 0;
  }
}

void orc_copcs_party_shares(int N, int64_t M, int64_t R, uint64_t *shares, uint64_t *random) {
  orc_copcs_party_shares_g(N, M, R, shares, random, NULL);
}

/* The same, and rank 0's generator as the dealing leaves it in *g_out (may
 * be NULL): nothing else draws from it until the leader's delegation. */
void orc_copcs_party_shares_g(int N, int64_t M, int64_t R, uint64_t *shares, uint64_t *random, orc_prng *g_out) {
  orc_prng g;
  orc_prng_seed(&g, 1); /* glibc's default state: the reference never seeds rank 0's generator */
  int64_t n = M > R ? M : R;
  uint64_t *buf = (uint64_t *)malloc(sizeof(uint64_t) * 2 * (size_t)(n ? n : 1));
  orc_generate_randomness(&g, M, buf);
  orc_secret_shares_g(buf, M, N, 1, &g, shares);
  orc_generate_randomness(&g, R, buf);
  orc_secret_shares_g(buf, R, N, 1, &g, random);
  free(buf);
  if (g_out) *g_out = g;
}

/* unpack_secret_share (MPI_utils.cpp:2769-2785) with _k = k = N */
static void unpack_all(uint64_t *sec, int N) {
  int lg = ilog2_64(N);
  orc_fft(sec, lg, 1, 1);
  fe w = f_inv(f_rou(1 + lg)), mul = f_one();
  for (int i = 0; i < N; i++) { st(sec, i, f_mul(mul, ld(sec, i))); mul = f_mul(w, mul); }
  orc_fft(sec, lg, 0, 1);
}

void orc_party_aggregate(const uint64_t *msgs, int N, int64_t len, const uint64_t *b, uint64_t *out) {
  uint64_t col[2 * 1024];
  for (int64_t i = 0; i < len; i++) {
    for (int p = 0; p < N; p++) { col[2 * p] = msgs[2 * (p * len + i)]; col[2 * p + 1] = msgs[2 * (p * len + i) + 1]; }
    unpack_all(col, N);
    fe acc = f_zero();
    for (int j = 0; j < N / 4; j++) acc = f_add(acc, f_mul(ld(b, j), ld(col, 2 * j)));
    st(out, i, acc);
  }
}

static void extend_block(const uint64_t *src, int logd, int ext_log, uint64_t *dst) {
  int64_t d = (int64_t)1 << logd, D = (int64_t)1 << (logd + ext_log);
  memset(dst, 0, sizeof(uint64_t) * 2 * D);
  memcpy(dst, src, sizeof(uint64_t) * 2 * d);
  orc_fft(dst, logd, 1, 1);
  orc_fft(dst, logd + ext_log, 0, 1);
}

void orc_cophase1(const uint64_t *p1, const uint64_t *p2, const uint64_t *p3, const uint64_t *b1, int64_t n,
                  int logd, uint64_t *H, uint64_t *H4) {
  int64_t d = (int64_t)1 << logd, blocks = n / d;
  uint64_t *a = (uint64_t *)malloc(sizeof(uint64_t) * 2 * 4 * d), *bb = (uint64_t *)malloc(sizeof(uint64_t) * 2 * 4 * d);
  uint64_t *c = (uint64_t *)malloc(sizeof(uint64_t) * 2 * 4 * d), *e = (uint64_t *)malloc(sizeof(uint64_t) * 2 * 4 * d);
  for (int64_t k = 0; k < 2 * d; k++) st(H, k, f_zero());
  for (int64_t k = 0; k < 4 * d; k++) st(H4, k, f_zero());
  for (int64_t j = 0; j < blocks; j++) {
    int zero = 1;
    for (int64_t k = 0; k < d; k++) if (p1[2 * (j * d + k)] || p1[2 * (j * d + k) + 1]) { zero = 0; break; }
    if (zero) continue;
    extend_block(p1 + 2 * j * d, logd, 1, a);
    extend_block(p2 + 2 * j * d, logd, 1, bb);
    for (int64_t k = 0; k < 2 * d; k++) st(H, k, f_add(ld(H, k), f_mul(ld(a, k), ld(bb, k))));
    extend_block(p1 + 2 * j * d, logd, 2, a);
    extend_block(p2 + 2 * j * d, logd, 2, bb);
    extend_block(b1 + 2 * j * d, logd, 2, c);
    extend_block(p3 + 2 * j * d, logd, 2, e);
    for (int64_t k = 0; k < 4 * d; k++)
      st(H4, k, f_add(ld(H4, k), f_mul(f_sub(f_mul(ld(a, k), ld(bb, k)), ld(e, k)), ld(c, k))));
  }
  free(a); free(bb); free(c); free(e);
}

void orc_cophase2(const uint64_t *v, int64_t n, const uint64_t *L, int logd, uint64_t *out) {
  int64_t d = (int64_t)1 << logd;
  for (int64_t j = 0; j < n / d; j++) {
    fe acc = f_zero();
    for (int64_t k = 0; k < d; k++) acc = f_add(acc, f_mul(ld(L, k), ld(v, j * d + k)));
    st(out, j, acc);
  }
}

/* ----------------------------------------- sumcheck round forms */
/* Line of a pair: linear_poly(v[2j+1] - v[2j], v[2j]) (polynomial.h:46-59). */
typedef struct { fe a, b; } lin_t;
static inline lin_t lin_at(const uint64_t *v, int64_t j) {
  fe lo = ld(v, 2 * j), hi = ld(v, 2 * j + 1);
  lin_t l = {f_sub(hi, lo), lo};
  return l;
}
/* linear * linear -> (a, b, c) (polynomial.cpp:133-135) */
static inline void lin_mul(lin_t x, lin_t y, fe q[3]) {
  q[0] = f_mul(x.a, y.a);
  q[1] = f_add(f_mul(x.a, y.b), f_mul(x.b, y.a));
  q[2] = f_mul(x.b, y.b);
}
/* quadratic * linear -> cubic (polynomial.cpp:91-93) */
static inline void quad_lin(const fe q[3], lin_t x, fe c[4]) {
  c[0] = f_mul(q[0], x.a);
  c[1] = f_add(f_mul(q[0], x.b), f_mul(q[1], x.a));
  c[2] = f_add(f_mul(q[1], x.b), f_mul(q[2], x.a));
  c[3] = f_mul(q[2], x.b);
}

/* cubic * linear -> quartic (polynomial.cpp:99-101) */
static inline void cub_lin(const fe c[4], lin_t x, fe q[5]) {
  q[0] = f_mul(c[0], x.a);
  q[1] = f_add(f_mul(c[1], x.a), f_mul(c[0], x.b));
  q[2] = f_add(f_mul(c[2], x.a), f_mul(c[1], x.b));
  q[3] = f_add(f_mul(c[3], x.a), f_mul(c[2], x.b));
  q[4] = f_mul(c[3], x.b);
}

int orc_sumcheck_form_vectors(int form) {
  static const int nv[5] = {2, 3, 6, 6, 4};
  return form >= 0 && form < 5 ? nv[form] : 0;
}
int orc_sumcheck_form_degree(int form) {
  static const int dg[5] = {2, 3, 2, 3, 4};
  return form >= 0 && form < 5 ? dg[form] : 0;
}

void orc_sumcheck_round(int form, const uint64_t *const *v, int64_t m, const uint64_t bb[2], uint64_t *out) {
  fe acc[5] = {f_zero(), f_zero(), f_zero(), f_zero(), f_zero()};
  fe accr[3] = {f_zero(), f_zero(), f_zero()};
  fe b = bb ? f_make(bb[0], bb[1]) : f_zero();
  for (int64_t j = 0; j < m / 2; j++) {
    fe q[3], c[4];
    if (form == 0) { /* coSumcheck_MPI.cpp:199 */
      lin_mul(lin_at(v[0], j), lin_at(v[1], j), q);
      for (int k = 0; k < 3; k++) acc[k] = f_add(acc[k], q[k]);
    } else if (form == 1) { /* Distributed_Sumcheck.cpp:1144-1151 */
      lin_mul(lin_at(v[0], j), lin_at(v[1], j), q);
      quad_lin(q, lin_at(v[2], j), c);
      for (int k = 0; k < 4; k++) acc[k] = f_add(acc[k], c[k]);
    } else if (form == 4) { /* quadruple_sumcheck, delegate_protocol.cpp:66-76 */
      fe q4[5];
      lin_mul(lin_at(v[0], j), lin_at(v[1], j), q);
      quad_lin(q, lin_at(v[2], j), c);
      cub_lin(c, lin_at(v[3], j), q4);
      for (int k = 0; k < 5; k++) acc[k] = f_add(acc[k], q4[k]);
    } else if (form == 2) { /* coSumcheck_MPI.cpp:156-176 */
      lin_mul(lin_at(v[0], j), lin_at(v[1], j), q);
      for (int k = 0; k < 3; k++) acc[k] = f_add(acc[k], q[k]);
      lin_mul(lin_at(v[2], j), lin_at(v[3], j), q);
      for (int k = 0; k < 3; k++) acc[k] = f_add(acc[k], q[k]);
      lin_mul(lin_at(v[4], j), lin_at(v[5], j), q);
      for (int k = 0; k < 3; k++) accr[k] = f_add(accr[k], q[k]);
    } else { /* coSumcheck_MPI.cpp:12-32: v = (v1, v2, v3, beta1, r1, r2) */
      fe qr[3];
      lin_mul(lin_at(v[0], j), lin_at(v[1], j), q);
      lin_mul(lin_at(v[4], j), lin_at(v[5], j), qr);
      lin_t l3 = lin_at(v[2], j);
      q[0] = f_add(q[0], f_mul(b, qr[0]));
      q[1] = f_sub(f_add(q[1], f_mul(b, qr[1])), l3.a);
      q[2] = f_sub(f_add(q[2], f_mul(b, qr[2])), l3.b);
      quad_lin(q, lin_at(v[3], j), c);
      for (int k = 0; k < 4; k++) acc[k] = f_add(acc[k], c[k]);
    }
  }
  if (form == 2)
    for (int k = 0; k < 3; k++) acc[k] = f_add(acc[k], f_mul(b, accr[k]));
  for (int k = 0; k <= orc_sumcheck_form_degree(form); k++) st(out, k, acc[k]);
}

void orc_sumcheck_fold_many(int nvec, uint64_t *const *v, int64_t m, const uint64_t r[2]) {
  fe rr = f_make(r[0], r[1]);
  for (int k = 0; k < nvec; k++)
    for (int64_t j = 0; j < m / 2; j++) {
      fe lo = ld(v[k], 2 * j), hi = ld(v[k], 2 * j + 1);
      st(v[k], j, f_add(lo, f_mul(rr, f_sub(hi, lo))));
    }
}

static fe cubic_eval(const fe c[4], fe x) {
  return f_add(f_mul(f_add(f_mul(f_add(f_mul(c[0], x), c[1]), x), c[2]), x), c[3]);
}

/* The distributed sumchecks of Distributed_Sumcheck.cpp for N parties held
 * in one process: form 0 is _quadratic_sumcheck (:204-349, vectors v1, v2),
 * form 1 is _cubic_sumcheck (:1122-1269, v1, v2, v3).  Party p owns entries
 * [p*M, (p+1)*M) of each vector.  Each of the log2(M) - offset rounds
 * combines the parties' round polynomials (a plain sum for form 0,
 * aggregate_poly :86-138; weights w[p] for form 1, :140-170), draws the
 * challenge hash_to_field of the coefficients from the chain fs
 * (prev_challenge) and folds every party's vectors.  The leader then runs
 * quadratic_sumcheck / cubic_sumcheck (sparse_eval.cpp:140-190, 419-475) over
 * the parties' remaining 2^offset entries gathered party by party (form 1
 * scales v3 by w[p], :1184-1189), taking the fourth F::_random() draw of each
 * round from the glibc stream g.  For form 0 with N > 1 the reference's
 * leader sizes its receive buffers for N parties each (:289-306) and so
 * reads zeros for the other parties' v2 entries, after which its consistency
 * check exits; the gathering here is the intended one, and parity with the
 * reference is defined for N = 1.
 * polys: (degree + 1) coefficients per round, chal: every challenge,
 * fin: the leader's v1[0], v2[0] (, v3[0]).  y is updated. */
void orc_party_sumcheck(int form, uint64_t *v1, uint64_t *v2, uint64_t *v3, int64_t M, int N, const uint64_t *w,
                        int offset, uint64_t fs[2], orc_prng *g, uint64_t y_io[2], uint64_t *polys,
                        uint64_t *chal, uint64_t *fin) {
  const int nv = form == 1 ? 3 : 2, nc = nv + 1;
  int lm = ilog2_64(M);
  int rounds = lm - offset;
  if (rounds <= 0) { rounds = 0; offset = lm; }
  fe y = f_make(y_io[0], y_io[1]);
  fe state = f_make(fs[0], fs[1]);
  int64_t cur = M;
  int r_i = 0;
  uint64_t *vv[3] = {v1, v2, v3};
  for (int i = 0; i < rounds; i++) {
    fe H[4] = {f_zero(), f_zero(), f_zero(), f_zero()};
    for (int p = 0; p < N; p++) {
      const uint64_t *pv[3];
      for (int k = 0; k < nv; k++) pv[k] = vv[k] + 2 * p * M;
      uint64_t c[8];
      orc_sumcheck_round(form, pv, cur, NULL, c);
      fe wp = form == 1 ? ld(w, p) : f_one();
      for (int k = 0; k < nc; k++) H[k] = f_add(H[k], form == 1 ? f_mul(wp, ld(c, k)) : ld(c, k));
    }
    for (int k = 0; k < nc; k++) st(polys, nc * r_i + k, H[k]);
    fe rnd = fs_absorb(&state, H, nc);
    st(chal, r_i, rnd);
    y = nc == 4 ? cubic_eval(H, rnd) : f_add(f_mul(f_add(f_mul(H[0], rnd), H[1]), rnd), H[2]);
    for (int p = 0; p < N; p++) {
      uint64_t *pv[3];
      for (int k = 0; k < nv; k++) pv[k] = vv[k] + 2 * p * M;
      orc_sumcheck_fold_many(nv, pv, cur, chal + 2 * r_i);
    }
    cur /= 2;
    r_i++;
  }
  int64_t S = (int64_t)1 << offset, T = S * N;
  uint64_t *gv[3] = {NULL, NULL, NULL};
  for (int k = 0; k < nv; k++) gv[k] = (uint64_t *)malloc(16 * T);
  for (int p = 0; p < N; p++)
    for (int64_t j = 0; j < S; j++)
      for (int k = 0; k < nv; k++) {
        fe x = ld(vv[k], p * M + j);
        if (k == 2) x = f_mul(ld(w, p), x);
        st(gv[k], p * S + j, x);
      }
  int lt = ilog2_64(T);
  for (int i = 0; i < lt; i++) {
    uint64_t c[8];
    orc_sumcheck_round(form, (const uint64_t *const *)gv, T >> i, NULL, c);
    for (int k = 0; k < nc; k++) st(polys, nc * r_i + k, ld(c, k));
    fe rnd = f_zero();
    for (int k = 0; k < 4; k++) rnd = prng_field(g);
    st(chal, r_i, rnd);
    const fe *cf = (const fe *)c;
    y = nc == 4 ? cubic_eval(cf, rnd) : f_add(f_mul(f_add(f_mul(cf[0], rnd), cf[1]), rnd), cf[2]);
    orc_sumcheck_fold_many(nv, gv, T >> i, chal + 2 * r_i);
    r_i++;
  }
  for (int k = 0; k < nv; k++) { fin[2 * k] = gv[k][0]; fin[2 * k + 1] = gv[k][1]; free(gv[k]); }
  fs[0] = state.re; fs[1] = state.im;
  y_io[0] = y.re; y_io[1] = y.im;
}

/* ------------------------------------------------ WHIR aggregation */
static fe dot(const uint64_t *a, const uint64_t *b, int64_t n) {
  fe acc = f_zero();
  for (int64_t t = 0; t < n; t++) acc = f_add(acc, f_mul(ld(a, t), ld(b, t)));
  return acc;
}

/* aggregate_claims (Whir.cpp:608-668) with every claim point of log2(n)
 * coordinates: betas_j = precompute_beta(point_j); Sums[i][j] =
 * <betas_j, arrays_i>; F::_random() draws c beta challenges then k array
 * challenges; K = sum_i sum_j bc_j ac_i Sums[i][j]; b_aggr = sum_j bc_j
 * betas_j; arr = sum_i ac_i arrays_i.  chal: the c + k challenges, sums: k*c
 * (row i = array). */
void orc_aggregate_claims(int k, const uint64_t *const *arrays, int64_t n, int c, const uint64_t *points,
                          orc_prng *g, uint64_t *arr, uint64_t *b_aggr, uint64_t K[2], uint64_t *chal,
                          uint64_t *sums) {
  int lg = ilog2_64(n);
  uint64_t *betas = (uint64_t *)malloc(16 * (size_t)n * (size_t)(c > 0 ? c : 1));
  for (int j = 0; j < c; j++) orc_precompute_beta(points + 2 * (size_t)j * lg, lg, betas + 2 * (size_t)j * n, 1);
  for (int i = 0; i < k; i++)
    for (int j = 0; j < c; j++) st(sums, (int64_t)i * c + j, dot(betas + 2 * (size_t)j * n, arrays[i], n));
  for (int j = 0; j < c + k; j++) st(chal, j, prng_field(g));
  fe Kacc = f_zero();
  for (int i = 0; i < k; i++)
    for (int j = 0; j < c; j++)
      Kacc = f_add(Kacc, f_mul(f_mul(ld(chal, j), ld(chal, c + i)), ld(sums, (int64_t)i * c + j)));
  K[0] = Kacc.re; K[1] = Kacc.im;
  for (int64_t t = 0; t < n; t++) {
    fe sb = f_zero(), sa = f_zero();
    for (int j = 0; j < c; j++) sb = f_add(sb, f_mul(ld(chal, j), ld(betas + 2 * (size_t)j * n, t)));
    for (int i = 0; i < k; i++) sa = f_add(sa, f_mul(ld(chal, c + i), ld(arrays[i], t)));
    st(b_aggr, t, sb);
    st(arr, t, sa);
  }
  free(betas);
}

/* aggregate_arrays (Whir.cpp:670-704): evals[i][j] = <arrays_i, B_j>;
 * arr += sum_{i>=1} r1_i arrays_i; b += sum_{i>=1} r2_i B_i; returns
 * K = sum_i sum_j r1_i r2_j evals[i][j].  Requires nB >= k. */
void orc_aggregate_arrays(uint64_t *arr, uint64_t *b, int k, const uint64_t *const *arrays, int nB,
                          const uint64_t *const *B, int64_t n, const uint64_t *r1, const uint64_t *r2, uint64_t K[2]) {
  fe Kacc = f_zero();
  for (int i = 0; i < k; i++)
    for (int j = 0; j < nB; j++)
      Kacc = f_add(Kacc, f_mul(f_mul(ld(r1, i), ld(r2, j)), dot(arrays[i], B[j], n)));
  for (int i = 1; i < k; i++)
    for (int64_t t = 0; t < n; t++) {
      st(arr, t, f_add(ld(arr, t), f_mul(ld(r1, i), ld(arrays[i], t))));
      st(b, t, f_add(ld(b, t), f_mul(ld(r2, i), ld(B[i], t))));
    }
  K[0] = Kacc.re; K[1] = Kacc.im;
}

/* aggregate_commitments (Whir.cpp:547-606): codeword = sum_i r_i cw_i; l
 * rand() draws for the (discarded) query openings, l as Whir.cpp:257; the
 * new tree has n/whir_k leaves, and since the loop that hashes the strided
 * leaf groups never stores its result (:594-601), every leaf is the zero
 * hash and the levels are those of create_tree_blake over zeros.  levels
 * gets 2 (n/whir_k) - 1 hashes, leaves first. */
void orc_aggregate_commitments(int k, const uint64_t *const *cws, int64_t n, const uint64_t *r, int rate, int whir_k,
                               orc_prng *g, uint64_t *codeword, uint8_t *levels) {
  for (int64_t t = 0; t < n; t++) {
    fe s = f_zero();
    for (int i = 0; i < k; i++) s = f_add(s, f_mul(ld(r, i), ld(cws[i], t)));
    st(codeword, t, s);
  }
  int l = orc_whir_queries(rate);
  for (int i = 0; i < l; i++) (void)orc_prng_next(g);
  int64_t leaves = n / whir_k;
  memset(levels, 0, 32 * (size_t)leaves);
  uint8_t *prev = levels;
  int64_t cnt = leaves;
  while (cnt > 1) {
    uint8_t *next = prev + 32 * cnt;
    cnt /= 2;
    for (int64_t i = 0; i < cnt; i++) hash_self(prev + 32 * (2 * i), next + 32 * i);
    prev = next;
  }
}

/* ------------------------------------------- coPCS open rounds */
/* tensor_eval_vector (coPCS.cpp:602-632): w1 = omega_{rate rows}^{p1},
 * w2 = omega_{4 cols}^{2 p0 + 1}; pow2[t] = w2^t (t < cols) goes through two
 * inverse transforms, is zero-padded to 2N = 4 cols and transformed; the
 * party my_id takes entry 2 my_id + 1 as its scale of B[j] = w1^j. */
void orc_tensor_eval_vector(uint32_t p0, uint32_t p1, int cols, int64_t rows, int rate, int my_id, uint64_t *B) {
  int N = 2 * cols;
  fe w1 = f_pow(f_rou(ilog2_64((int64_t)rate * rows)), (u128)p1);
  fe w2 = f_pow(f_rou(ilog2_64(4 * (int64_t)cols)), (u128)(2 * (uint64_t)p0 + 1));
  uint64_t *buf = (uint64_t *)calloc(2 * 2 * (size_t)N, sizeof(uint64_t));
  fe x = f_one();
  for (int t = 0; t < cols; t++) { st(buf, t, x); x = f_mul(x, w2); }
  orc_fft(buf, ilog2_64(cols), 1, 1);
  orc_fft(buf, ilog2_64(cols), 1, 1);
  orc_fft(buf, ilog2_64(2 * N), 0, 1);
  fe c = ld(buf, 2 * my_id + 1);
  free(buf);
  fe y = c;
  for (int64_t j = 0; j < rows; j++) { st(B, j, y); y = f_mul(y, w1); }
}

/* pcs_sumcheck_phase3 (coPCS.cpp:634-648): B += sum_i s^{i+1}
 * tensor_eval_vector(query_i); queries: l pairs (point[0], point[1]). */
void orc_pcs_phase3(uint64_t *B, int64_t rows, const uint32_t *queries, int l, const uint64_t s[2], int N, int rate,
                    int my_id) {
  fe ss = f_make(s[0], s[1]), p = ss;
  uint64_t *tmp = (uint64_t *)malloc(16 * (size_t)rows);
  for (int i = 0; i < l; i++) {
    orc_tensor_eval_vector(queries[2 * i], queries[2 * i + 1], N / 2, rows, rate, my_id, tmp);
    for (int64_t j = 0; j < rows; j++) st(B, j, f_add(ld(B, j), f_mul(p, ld(tmp, j))));
    p = f_mul(p, ss);
  }
  free(tmp);
}

/* encode_concatenated (coPCS.cpp:653-677): C' = forward transform of the
 * data zero-padded to rate0 * n (L entries); column j < L/degree gathers
 * C'[j + k L/degree] for k < degree, is zero-padded to degree * rate1 and
 * transformed.  C: L/degree rows of degree * rate1 entries. */
void orc_encode_concatenated(const uint64_t *data, int64_t n, int rate0, int rate1, int degree, uint64_t *Cprime,
                             uint64_t *C) {
  int64_t L = n * rate0, rows = L / degree, D = (int64_t)degree * rate1;
  memset(Cprime, 0, 16 * (size_t)L);
  memcpy(Cprime, data, 16 * (size_t)n);
  orc_fft(Cprime, ilog2_64(L), 0, 0);
  for (int64_t j = 0; j < rows; j++) {
    uint64_t *row = C + 2 * j * D;
    memset(row, 0, 16 * (size_t)D);
    for (int k = 0; k < degree; k++) st(row, k, ld(Cprime, j + k * rows));
    orc_fft(row, ilog2_64(D), 0, 1);
  }
}

/* ================================================ Whir_Batch_Open */
/* Whir_Batch_Open (Whir.cpp:706-898) opens k polynomials of non-increasing
 * sizes: the largest is folded by WHIR iterations, and whenever it reaches
 * the size of the next ones they are merged into it (aggregate_arrays,
 * aggregate_commitments).  bo_make_plan restates the control flow on the
 * sizes alone: the kappa schedule of Whir.cpp:731-752 and the loop of
 * :761-833, including the schedule read at :819-822 (whir_k =
 * kappas[iter + 1] after iter was advanced).  Inputs on which the reference
 * reads past its schedule or opens a Merkle leaf beyond the tree (it exits
 * in open_tree_blake) are rejected. */
#define BO_MAX_STEPS 64
typedef struct {
  int iterate, kappa;              /* a WHIR iteration folding by kappa */
  int aggregate, group, first;     /* merge arrays first .. first+group-2 into the current one */
  int64_t m, L;                    /* sizes when the step starts */
  int rate;                        /* rate when the step starts */
  int l, depth;                    /* iteration: queries, path length in the current tree */
  int la, depth_a;                 /* aggregation: queries, path length */
  int64_t leaves_after;            /* leaves of the tree the step leaves behind */
} bo_exec;
typedef struct {
  int nsched, nexec;
  int32_t kappa[BO_MAX_STEPS], aggr[BO_MAX_STEPS];
  bo_exec ex[BO_MAX_STEPS];
  int64_t m_final;
  int64_t cw_len[64];
  int64_t bytes;
} bo_plan;

static int is_p2(int64_t x) { return x > 0 && (x & (x - 1)) == 0; }

static int bo_make_plan(int k, const int64_t *sizes, int rate, int whir_k, bo_plan *P) {
  memset(P, 0, sizeof(*P));
  if (k < 1 || k > 64) return -1;
  if (!(whir_k == 2 || whir_k == 4 || whir_k == 8 || whir_k == 16)) return -1;
  if (rate < 2 || !is_p2(rate)) return -1;
  for (int i = 0; i < k; i++) {
    if (!is_p2(sizes[i])) return -1;
    if (i && sizes[i] > sizes[i - 1]) return -1;
  }
  if (sizes[0] < 2 * whir_k || ilog2_64(sizes[0] * rate) > 28) return -1;
  /* kappa schedule (Whir.cpp:731-752) */
  int64_t size = sizes[0];
  int si = 1;
  for (;;) {
    if (P->nsched >= BO_MAX_STEPS) return -1;
    if (si >= k || size / whir_k > sizes[si]) {
      P->kappa[P->nsched] = whir_k;
      P->aggr[P->nsched++] = 0;
      size /= whir_k;
    } else {
      int64_t kap = size / sizes[si];
      int64_t s = sizes[si];
      while (si < k && sizes[si] == s) si++;
      P->kappa[P->nsched] = (int32_t)kap;
      P->aggr[P->nsched++] = 1;
      size /= kap;
    }
    if (size <= whir_k) break;
  }
  /* main loop (Whir.cpp:761-833) */
  int64_t m = sizes[0], L = m * rate, leaves = L / 4;
  int cur = rate, iter = 0, next = 1, wk = whir_k;
  int64_t bytes = 8 + 8 * (int64_t)P->nsched;
  P->cw_len[0] = L;
  for (;;) {
    if (iter >= P->nsched || P->nexec >= BO_MAX_STEPS) return -1;
    bo_exec *e = &P->ex[P->nexec++];
    wk = P->kappa[iter];
    int ag = P->aggr[iter];
    e->m = m;
    e->L = L;
    e->rate = cur;
    if (!ag || wk != 1) {
      int kap = wk, logk = ilog2_64(kap);
      if (kap < 2 || m < kap) return -1;
      int64_t qmod = kap > 4 ? L / kap : L / 4;
      if (qmod > leaves) return -1; /* open_tree_blake would exit */
      e->iterate = 1;
      e->kappa = kap;
      e->l = orc_whir_queries(cur);
      e->depth = ilog2_64(leaves);
      int64_t nm = m / kap, NL = 2 * (int64_t)cur * nm;
      if (NL < 8 || e->l > 256) return -1;
      bytes += (int64_t)logk * (8 + 48 + 8 + 16) + (8 + 32) + (8 + 4 * (int64_t)e->l) +
               (8 + 16 * (int64_t)kap * e->l) + (8 + 16 * (int64_t)e->l) + (8 + 32 * (int64_t)e->l * e->depth) +
               (8 + 16 * (int64_t)e->l) + (8 + 16);
      m = nm;
      L = NL;
      leaves = L / 4;
      cur *= 2;
    }
    iter++;
    if (ag) {
      int g = 1;
      while (next + g - 1 < k && sizes[next + g - 1] == m) g++;
      e->aggregate = 1;
      e->group = g;
      e->first = next;
      for (int i = 0; i < g - 1; i++) P->cw_len[next + i] = L;
      next += g - 1;
      if (iter + 1 >= P->nsched) return -1; /* kappas[iter + 1] past the schedule */
      int64_t wk2 = P->kappa[iter + 1];
      if (next < k && m / wk2 <= sizes[next]) wk2 = m / sizes[next];
      if (wk2 < 1 || L % wk2 || leaves != L / 4) return -1;
      e->la = orc_whir_queries((int)(L / m));
      e->depth_a = ilog2_64(leaves);
      if (e->la > 256) return -1;
      leaves = L / wk2;
      wk = (int)wk2;
      bytes += (8 + 32 * (int64_t)g) + (8 + 16) + (8 + 4 * (int64_t)e->la) + (8 + 32 * (int64_t)e->la * e->depth_a) +
               (8 + 32);
    }
    e->leaves_after = leaves;
    if (m <= wk) break;
  }
  P->m_final = m;
  bytes += (8 + 16 * m) + (8 + 16 * (int64_t)ilog2_64(m)) + (8 + 16);
  P->bytes = bytes;
  return 0;
}

int orc_whir_batch_schedule(int k, const int64_t *sizes, int rate, int whir_k, int32_t *kappa, int32_t *aggr,
                            int64_t *cw_len, int64_t *bytes) {
  bo_plan P;
  if (bo_make_plan(k, sizes, rate, whir_k, &P) < 0) return -1;
  for (int i = 0; i < P.nsched; i++) {
    if (kappa) kappa[i] = P.kappa[i];
    if (aggr) aggr[i] = P.aggr[i];
  }
  for (int i = 0; i < k; i++)
    if (cw_len) cw_len[i] = P.cw_len[i];
  if (bytes) *bytes = P.bytes;
  return P.nsched;
}

/* open_tree_blake (merkle_tree.cpp:320-335) over a tree of `leaves` leaf hashes. */
static void bo_open(const uint8_t *levels, int64_t leaves, int64_t pos, uint8_t *out) {
  const uint8_t *lv = levels;
  int64_t cnt = leaves;
  int d = 0;
  while (cnt > 1) {
    memcpy(out + 32 * d, lv + 32 * (pos ^ 1), 32);
    d++;
    lv += 32 * cnt;
    cnt /= 2;
    pos /= 2;
  }
}

/* The transcript of the batch opening: SCHEDULE, then per executed step the
 * WHIR iteration records (as in orc_prove, with kappa replies per query)
 * and/or the aggregation records AGGR_CHALLENGES (the draws of Whir.cpp:809-814
 * after the [0] = 1 overrides), AGGR_K (aggregate_arrays), AGGR_QUERIES and
 * AGGR_PATHS (the openings of aggregate_commitments, Whir.cpp:574-585) and
 * AGGR_ROOT (the tree over zero leaves it installs, :594-604); last the
 * final polynomial, point and evaluation (Whir.cpp:840-869).  *check_ok
 * (optional) receives whether K equals sum arr * b at the end
 * (verification step 2, Whir.cpp:848-855). */
enum { T_SCHEDULE = 19, T_AGGR_CHALLENGES = 20, T_AGGR_K = 21, T_AGGR_QUERIES = 22, T_AGGR_PATHS = 23,
       T_AGGR_ROOT = 24 };

int64_t orc_whir_batch_open(int k, const uint64_t *const *arrays, const int64_t *sizes,
                            const uint64_t *const *codewords, const uint8_t *levels0, const uint64_t *const *betas,
                            const uint64_t K0[2], int rate, int whir_k, orc_prng *g, uint8_t *transcript,
                            int64_t cap, int *check_ok, int threads) {
  bo_plan P;
  if (bo_make_plan(k, sizes, rate, whir_k, &P) < 0) return -1;
  tw_t tw = {transcript, 0, cap, 0};
  {
    uint32_t sch[2 * BO_MAX_STEPS];
    for (int i = 0; i < P.nsched; i++) {
      sch[2 * i] = (uint32_t)P.kappa[i];
      sch[2 * i + 1] = (uint32_t)P.aggr[i];
    }
    tw_raw(&tw, T_SCHEDULE, sch, (uint32_t)(2 * P.nsched), 4);
  }
  int64_t n0 = sizes[0];
  fe *arr = (fe *)malloc(sizeof(fe) * (size_t)n0), *b = (fe *)malloc(sizeof(fe) * (size_t)n0);
  memcpy(arr, arrays[0], sizeof(fe) * (size_t)n0);
  memcpy(b, betas[0], sizeof(fe) * (size_t)n0);
  int64_t L = n0 * rate, m = n0, leaves = L / 4;
  fe *cw = (fe *)malloc(sizeof(fe) * (size_t)L);
  memcpy(cw, codewords[0], sizeof(fe) * (size_t)L);
  uint8_t *tree = (uint8_t *)malloc((size_t)32 * (size_t)(2 * leaves));
  memcpy(tree, levels0, (size_t)32 * (size_t)(2 * leaves - 1));
  fe K = f_make(K0[0], K0[1]);
  int cur = rate;
  for (int s = 0; s < P.nexec; s++) {
    const bo_exec *e = &P.ex[s];
    if (e->iterate) {
      const int kap = e->kappa, logk = ilog2_64(kap);
      fe r[4];
      for (int i = 0; i < logk; i++) { /* whir_sumcheck (Whir.cpp:233-249) */
        uint64_t H6[6];
        orc_sumcheck_quadratic((const uint64_t *)arr, (const uint64_t *)b, m, H6, threads);
        fe h[3] = {f_make(H6[0], H6[1]), f_make(H6[2], H6[3]), f_make(H6[4], H6[5])};
        tw_fe(&tw, T_WHIR_POLY, h, 3);
        r[i] = prng_field(g);
        tw_fe(&tw, T_WHIR_CHALLENGE, &r[i], 1);
        K = quad_eval(h, r[i]);
        uint64_t c2[2] = {r[i].re, r[i].im};
        orc_sumcheck_fold((uint64_t *)arr, m, c2, threads);
        orc_sumcheck_fold((uint64_t *)b, m, c2, threads);
        m /= 2;
      }
      fe *ncw;
      uint8_t *ntree;
      whir_commit(arr, m, 2 * cur, &ncw, &ntree, threads);
      int64_t NL = m * 2 * cur;
      tw_raw(&tw, T_WHIR_ROOT, tree_root(ntree, NL), 1, 32);
      /* whir_query (Whir.cpp:251-314) on the current codeword and tree */
      const int l = e->l;
      const int64_t qmod = kap > 4 ? L / kap : L / 4;
      int32_t *q = (int32_t *)malloc(sizeof(int32_t) * (size_t)l);
      for (int i = 0; i < l; i++) q[i] = orc_prng_next(g) % (int32_t)qmod;
      tw_raw(&tw, T_WHIR_QUERIES, q, (uint32_t)l, 4);
      fe *rep = (fe *)malloc(sizeof(fe) * (size_t)l * kap), *ans = (fe *)malloc(sizeof(fe) * (size_t)l);
      for (int i = 0; i < l; i++) {
        for (int j = 0; j < kap; j++) rep[i * kap + j] = cw[q[i] + j * (L / kap)];
        ans[i] = rs_fold_tensor(rep + (int64_t)i * kap, logk, r, L, q[i]);
      }
      tw_fe(&tw, T_WHIR_REPLIES, rep, (uint32_t)(l * kap));
      tw_fe(&tw, T_WHIR_ANSWERS, ans, (uint32_t)l);
      uint8_t *paths = (uint8_t *)malloc((size_t)32 * (size_t)l * (size_t)(e->depth > 0 ? e->depth : 1));
      for (int i = 0; i < l; i++) bo_open(tree, leaves, q[i], paths + (size_t)32 * e->depth * i);
      tw_raw(&tw, T_WHIR_PATHS, paths, (uint32_t)(l * e->depth), 32);
      free(paths);
      free(rep);
      for (int i = 0; i < l; i++) q[i] = q[i] * (int32_t)(kap * NL / L); /* Whir.cpp:371-372 */
      free(cw);
      free(tree);
      cw = ncw;
      tree = ntree;
      L = NL;
      leaves = L / 4;
      fe rb = prng_field(g);
      fe *ch = (fe *)malloc(sizeof(fe) * (size_t)l);
      uint64_t rb2[2] = {rb.re, rb.im};
      orc_update_betas((uint64_t *)b, m, q, l, L, rb2, (uint64_t *)ch, threads);
      tw_fe(&tw, T_WHIR_COMBINE, ch, (uint32_t)l);
      for (int i = 0; i < l; i++) K = f_add(K, f_mul(ch[i], ans[i]));
      tw_fe(&tw, T_WHIR_K, &K, 1);
      free(ch);
      free(ans);
      free(q);
      cur *= 2;
    }
    if (e->aggregate) {
      const int gsz = e->group;
      fe *ch = (fe *)malloc(sizeof(fe) * 2 * (size_t)gsz); /* ch1 then ch2 */
      for (int i = 0; i < 2 * gsz; i++) ch[i] = prng_field(g);
      ch[0] = f_one();
      ch[gsz] = f_one();
      tw_fe(&tw, T_AGGR_CHALLENGES, ch, (uint32_t)(2 * gsz));
      const fe *c1 = ch, *c2 = ch + gsz;
      /* aggregate_arrays(arr, b, arr_aggr, B_aggr, r1 = ch2, r2 = ch1) (Whir.cpp:670-703) */
      const fe **A = (const fe **)malloc(sizeof(fe *) * (size_t)gsz), **B = (const fe **)malloc(sizeof(fe *) * (size_t)gsz);
      fe *a0 = (fe *)malloc(sizeof(fe) * (size_t)m), *b0 = (fe *)malloc(sizeof(fe) * (size_t)m);
      memcpy(a0, arr, sizeof(fe) * (size_t)m);
      memcpy(b0, b, sizeof(fe) * (size_t)m);
      A[0] = a0;
      B[0] = b0;
      for (int i = 1; i < gsz; i++) {
        A[i] = (const fe *)arrays[e->first + i - 1];
        B[i] = (const fe *)betas[e->first + i - 1];
      }
      fe Kn = f_zero();
      for (int i = 0; i < gsz; i++)
        for (int j = 0; j < gsz; j++) {
          fe d = f_zero();
          for (int64_t t = 0; t < m; t++) d = f_add(d, f_mul(A[i][t], B[j][t]));
          Kn = f_add(Kn, f_mul(f_mul(c2[i], c1[j]), d));
        }
      for (int i = 1; i < gsz; i++)
        for (int64_t t = 0; t < m; t++) {
          arr[t] = f_add(arr[t], f_mul(c2[i], A[i][t]));
          b[t] = f_add(b[t], f_mul(c1[i], B[i][t]));
        }
      K = Kn;
      tw_fe(&tw, T_AGGR_K, &K, 1);
      /* aggregate_commitments(codeword, MT, codewords_aggr, MT_aggr, ch2, L / m) (Whir.cpp:547-606) */
      fe *ncw = (fe *)malloc(sizeof(fe) * (size_t)L);
      for (int64_t t = 0; t < L; t++) {
        fe acc = f_mul(c2[0], cw[t]);
        for (int i = 1; i < gsz; i++) acc = f_add(acc, f_mul(c2[i], ld(codewords[e->first + i - 1], t)));
        ncw[t] = acc;
      }
      const int la = e->la;
      int32_t *qa = (int32_t *)malloc(sizeof(int32_t) * (size_t)la);
      for (int i = 0; i < la; i++) qa[i] = orc_prng_next(g) % (int32_t)(L / 4);
      tw_raw(&tw, T_AGGR_QUERIES, qa, (uint32_t)la, 4);
      uint8_t *paths = (uint8_t *)malloc((size_t)32 * (size_t)la * (size_t)(e->depth_a > 0 ? e->depth_a : 1));
      for (int i = 0; i < la; i++) bo_open(tree, leaves, qa[i], paths + (size_t)32 * e->depth_a * i);
      tw_raw(&tw, T_AGGR_PATHS, paths, (uint32_t)(la * e->depth_a), 32);
      free(paths);
      free(qa);
      const int64_t nleaves = e->leaves_after;
      uint8_t *ztree = (uint8_t *)calloc((size_t)(2 * nleaves), 32);
      {
        uint8_t *prev = ztree;
        int64_t cnt = nleaves;
        while (cnt > 1) {
          uint8_t *nxt = prev + 32 * cnt;
          cnt /= 2;
          for (int64_t i = 0; i < cnt; i++) hash_self(prev + 32 * (2 * i), nxt + 32 * i);
          prev = nxt;
        }
        tw_raw(&tw, T_AGGR_ROOT, prev, 1, 32);
      }
      free(cw);
      free(tree);
      cw = ncw;
      tree = ztree;
      leaves = nleaves;
      free(a0);
      free(b0);
      free(A);
      free(B);
      free(ch);
    }
  }
  /* final round (Whir.cpp:840-869) */
  tw_fe(&tw, T_FINAL_POLY, arr, (uint32_t)m);
  fe Kc = K;
  for (int64_t t = 0; t < m; t++) Kc = f_sub(Kc, f_mul(arr[t], b[t]));
  if (check_ok) *check_ok = f_eq(Kc, f_zero());
  int lgm = ilog2_64(m);
  fe rf[8];
  for (int i = 0; i < lgm; i++) rf[i] = prng_field(g);
  tw_fe(&tw, T_FINAL_POINT, rf, (uint32_t)lgm);
  uint64_t ev[2];
  orc_evaluate_vector((const uint64_t *)b, m, (const uint64_t *)rf, ev);
  fe e = f_make(ev[0], ev[1]);
  tw_fe(&tw, T_FINAL_EVAL, &e, 1);
  free(arr);
  free(b);
  free(cw);
  free(tree);
  return tw.bad ? -1 : tw.len;
}
