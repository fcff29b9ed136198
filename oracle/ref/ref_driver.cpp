// Single-process driver over the reference prover's own functions.
//
// Test infrastructure only.  It links the unmodified reference sources
// (oracle/ref/Makefile) and writes golden vectors that pin the C restatement
// in oracle/gbz_oracle.c and, through it, the CUDA path.  Every subcommand
// calls reference functions; the only logic written here is input
// generation, the call order, and serialisation of what the reference
// returns.
//
//   ref_driver field   <count> <seed>              > out
//   ref_driver blake3  <count> <seed>              > out
//   ref_driver fft     <logn> <inverse> <seed>     > out   (fft, utils.cpp:904)
//   ref_driver pfft    <logn> <seed>               > out   (pfft, utils.cpp:1583)
//   ref_driver merkle  <logN> <seed>               > out   (MT_commit_Blake, merkle_tree.cpp:195)
//   ref_driver fs      <count> <seed>              > out   (hash_to_field, Fiat_Shamir.cpp:29)
//   ref_driver prng    <count> <seed>              > out   (F::_random, fieldElement.cpp:119)
//   ref_driver beta    <logn> <seed>               > out   (precompute_beta, utils.cpp:198)
//   ref_driver tensor  <logn> <logk> <count> <seed> > out  (get_RS_multifold_segment_tensor, coPCS_utils.cpp:333)
//   ref_driver betas   <logb> <logN> <l> <seed> <prng_seed> > out (update_betas, Whir.cpp:325)
//   ref_driver prove   <logn> <rate> <seed> <prng_seed> > transcript
//
// Witness/input generation: SplitMix64(seed); a base-field value takes the
// top 61 bits of one output and rejects the single value p.
#include "config_pc.hpp"
#include "utils.hpp"
#include "merkle_tree.h"
#include "Fiat_Shamir.h"
#include "polynomial.h"
#include "Whir.h"
#include "coPCS_utils.h"
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using std::vector;

// Reference functions defined in Whir.cpp without a header declaration.
quadratic_poly whir_sumcheck_step1(vector<F> &arr, vector<F> &b);
void whir_sumcheck_step2(vector<F> &arr, vector<F> &b, F c);
vector<F> whir_query(vector<F> &codeword, vector<vector<_hash>> &MT, vector<F> r,
                     vector<int> &queries, int rate);
vector<F> update_betas(vector<F> &b, vector<int> queries, int n);
extern F prev_challenge;

static const uint64_t P61 = 2305843009213693951ULL;

struct SplitMix {
  uint64_t s;
  explicit SplitMix(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  uint64_t base() {
    for (;;) {
      uint64_t v = next() >> 3;
      if (v != P61) return v;
    }
  }
  F elem_base() { F x; x.real = base(); x.img = 0; return x; }
  F elem_ext() { F x; x.real = base(); x.img = base(); return x; }
};

static void put(const void *p, size_t n) { fwrite(p, 1, n, stdout); }
static void putF(const F &x) { put(&x.real, 8); put(&x.img, 8); }
static void putFs(const vector<F> &v) { for (auto &x : v) putF(x); }

// Transcript record: u32 tag, u32 count, then count units.
static void rec(uint32_t tag, uint32_t count, const void *payload, size_t unit) {
  put(&tag, 4); put(&count, 4); put(payload, unit * count);
}
static void recF(uint32_t tag, const vector<F> &v) {
  uint32_t c = (uint32_t)v.size(); put(&tag, 4); put(&c, 4); putFs(v);
}

enum {
  T_COMMIT_ROOT = 1, T_EVAL_POINT = 2, T_CLAIM = 3, T_SC_POLY = 4, T_SC_CHALLENGE = 5,
  T_SC_FINAL = 6, T_WHIR_POLY = 7, T_WHIR_CHALLENGE = 8, T_WHIR_ROOT = 9,
  T_WHIR_QUERIES = 10, T_WHIR_REPLIES = 11, T_WHIR_ANSWERS = 12, T_WHIR_PATHS = 13,
  T_WHIR_COMBINE = 14, T_WHIR_K = 15, T_FINAL_POLY = 16, T_FINAL_POINT = 17,
  T_FINAL_EVAL = 18
};

static int cmd_field(int count, uint64_t seed) {
  SplitMix g(seed);
  vector<F> a, b;
  // edge values first: 0, 1, p-1, small, 2^60, the root-of-unity generator
  const uint64_t edges[] = {0, 1, P61 - 1, 2, 1ULL << 60, 2147483648ULL, 1033321771269002680ULL};
  for (uint64_t x : edges) for (uint64_t y : edges) {
    F u, v; u.real = x; u.img = y; v.real = y; v.img = x; a.push_back(u); b.push_back(v);
  }
  for (int i = 0; i < count; i++) { a.push_back(g.elem_ext()); b.push_back(g.elem_ext()); }
  uint32_t n = (uint32_t)a.size();
  put(&n, 4);
  for (uint32_t i = 0; i < n; i++) {
    putF(a[i]); putF(b[i]);
    putF(a[i] + b[i]); putF(a[i] - b[i]); putF(a[i] * b[i]); putF(-a[i]);
    putF(a[i].inv());
  }
  for (int lg = 0; lg <= 61; lg++) putF(getRootOfUnity(lg));
  return 0;
}

static int cmd_blake3(int count, uint64_t seed) {
  SplitMix g(seed);
  uint32_t n = (uint32_t)count;
  put(&n, 4);
  for (int i = 0; i < count; i++) {
    uint8_t in[64], out[32];
    for (int j = 0; j < 8; j++) { uint64_t w = g.next(); memcpy(in + 8 * j, &w, 8); }
    if (i == 0) memset(in, 0, 64);
    blake3_hash(in, out);
    put(in, 64); put(out, 32);
  }
  return 0;
}

static int cmd_fft(int logn, int inverse, uint64_t seed, bool use_pfft) {
  SplitMix g(seed);
  vector<F> a(1u << logn);
  for (auto &x : a) x = g.elem_ext();
  vector<F> out = a;
  if (use_pfft) pfft(out, logn, false);
  else fft(out, logn, inverse != 0);
  putFs(a); putFs(out);
  return 0;
}

static int cmd_merkle(int logN, uint64_t seed) {
  SplitMix g(seed);
  vector<F> a(1u << logN);
  for (auto &x : a) x = g.elem_ext();
  vector<vector<_hash>> mt;
  merkle_tree::merkle_tree_prover::MT_commit_Blake(a.data(), mt, (int)a.size());
  putFs(a);
  uint32_t lv = (uint32_t)mt.size();
  put(&lv, 4);
  for (auto &level : mt) {
    uint32_t c = (uint32_t)level.size();
    put(&c, 4);
    for (auto &h : level) put(h.arr, 32);
  }
  return 0;
}

static int cmd_fs(int count, uint64_t seed) {
  SplitMix g(seed);
  prev_challenge = F(0);
  vector<F> in(count);
  for (auto &x : in) x = g.elem_ext();
  vector<F> out;
  // absorb in groups of 1, 2 and 3 elements like the reference callers do
  int i = 0, grp = 1;
  while (i < count) {
    vector<F> chunk;
    for (int k = 0; k < grp && i < count; k++) chunk.push_back(in[i++]);
    out.push_back(hash_to_field(chunk));
    grp = grp % 3 + 1;
  }
  vector<vector<u32>> idx = get_indexes(8, 1 << 10, 1 << 12, -1);
  putFs(in); putFs(out);
  for (auto &v : idx) { put(&v[0], 4); put(&v[1], 4); }
  putF(prev_challenge);
  return 0;
}

static int cmd_prng(int count, unsigned prng_seed) {
  srandom(prng_seed);
  for (int i = 0; i < count; i++) putF(F::_random());
  for (int i = 0; i < 16; i++) { int q = rand(); put(&q, 4); }
  return 0;
}

static int cmd_beta(int logn, uint64_t seed) {
  SplitMix g(seed);
  vector<F> r(logn);
  for (auto &x : r) x = g.elem_ext();
  vector<F> B;
  precompute_beta(r, B);
  vector<F> v(1u << logn);
  for (auto &x : v) x = g.elem_ext();
  F e = evaluate_vector(v, r);
  vector<F> r2(logn);
  for (auto &x : r2) x = g.elem_ext();
  F bi = beta_identity(r, r2);
  putFs(r); putFs(B); putFs(v); putF(e); putFs(r2); putF(bi);
  return 0;
}

static int cmd_tensor(int logn, int logk, int count, uint64_t seed) {
  SplitMix g(seed);
  int n = 1 << logn, k = 1 << logk;
  uint32_t c = (uint32_t)count;
  put(&c, 4);
  for (int t = 0; t < count; t++) {
    vector<F> seg(k), r(logk);
    for (auto &x : seg) x = g.elem_ext();
    for (auto &x : r) x = g.elem_ext();
    int idx = (int)(g.next() % (uint64_t)(n / k));
    F y = get_RS_multifold_segment_tensor(seg, r, n, idx);
    put(&idx, 4); putFs(seg); putFs(r); putF(y);
  }
  return 0;
}

static int cmd_betas(int logb, int logN, int l, uint64_t seed, unsigned prng_seed) {
  SplitMix g(seed);
  vector<F> b(1u << logb);
  for (auto &x : b) x = g.elem_ext();
  vector<int> q(l);
  for (auto &x : q) x = (int)(g.next() % (1ULL << logN));
  putFs(b);
  for (int x : q) put(&x, 4);
  srandom(prng_seed);
  vector<F> ch = update_betas(b, q, 1 << logN);
  putFs(ch); putFs(b);
  return 0;
}

// The plain single-party prover: commit (Whir_Commit_initial), the evaluation
// point from the Fiat-Shamir chain (main.cpp:83-85), one quadratic sumcheck
// with Fiat-Shamir challenges (the round body of _quadratic_cosumcheck,
// coSumcheck_MPI.cpp:195-219, at one party), then the WHIR opening of the
// resulting claim (Whir_Open, Whir.cpp:388-467) with whir_k = 4.  The WHIR
// part is driven through the reference's own step functions so that each
// round's message can be written out; `check` then re-runs the unmodified
// Whir_Open on copies from the same PRNG state and compares.
static int cmd_prove(int logn, int rate, uint64_t seed, unsigned prng_seed, bool check) {
  whir_k = 4;
  SplitMix g(seed);
  const int n = 1 << logn;
  vector<F> w(n);
  for (auto &x : w) x = g.elem_base();

  srandom(prng_seed);
  prev_challenge = F(0);

  // 1. commitment
  vector<F> codeword;
  vector<vector<_hash>> MT;
  Whir_Commit_initial(w, codeword, MT, rate, whir_k);
  rec(T_COMMIT_ROOT, 1, MT.back()[0].arr, 32);

  // 2. evaluation point
  vector<F> z;
  for (int i = 0; i < logn; i++) z.push_back(hash_to_field({F(0)}));
  recF(T_EVAL_POINT, z);
  vector<F> beta;
  precompute_beta(z, beta);
  F y = F(0);
  for (int i = 0; i < n; i++) y += w[i] * beta[i];
  recF(T_CLAIM, {y});

  // 3. sumcheck of sum_x w(x) * eq(z, x)
  vector<F> v1 = w, v2 = beta, chal(logn);
  for (int i = 0; i < logn; i++) {
    quadratic_poly H(F_ZERO, F_ZERO, F_ZERO);
    for (int j = 0; j < (int)v1.size() / (1 << (i + 1)); j++)
      H = H + linear_poly(v1[2 * j + 1] - v1[2 * j], v1[2 * j]) *
                  linear_poly(v2[2 * j + 1] - v2[2 * j], v2[2 * j]);
    if (H.eval(0) + H.eval(1) != y) { fprintf(stderr, "sumcheck round %d inconsistent\n", i); return 2; }
    recF(T_SC_POLY, {H.a, H.b, H.c});
    chal[i] = hash_to_field({H.a, H.b, H.c});
    recF(T_SC_CHALLENGE, {chal[i]});
    y = H.eval(chal[i]);
    for (int j = 0; j < (int)v1.size() / (1 << (i + 1)); j++) {
      v1[j] = chal[i] * (v1[2 * j + 1] - v1[2 * j]) + v1[2 * j];
      v2[j] = chal[i] * (v2[2 * j + 1] - v2[2 * j]) + v2[2 * j];
    }
  }
  recF(T_SC_FINAL, {v1[0], v2[0]});

  // Snapshot for the unmodified Whir_Open run.
  vector<F> w_copy = w, cw_copy = codeword;
  vector<vector<_hash>> MT_copy = MT;
  char prng_snapshot[256];
  static char statebuf[128];
  (void)prng_snapshot;
  // glibc keeps one global generator; replay it by reseeding and skipping
  // the draws made so far (none before WHIR in this pipeline).

  // 4. WHIR open of (v1[0], chal)
  F K = v1[0];
  vector<F> b;
  precompute_beta(chal, b);
  vector<F> arr = w;
  int cur_rate = rate;
  while (true) {
    vector<F> r;
    for (int i = 0; i < (int)log2(whir_k); i++) {
      quadratic_poly h = whir_sumcheck_step1(arr, b);
      if (K != h.eval(F(0)) + h.eval(F(1))) { fprintf(stderr, "whir sumcheck inconsistent\n"); return 2; }
      recF(T_WHIR_POLY, {h.a, h.b, h.c});
      r.push_back(F::_random());
      recF(T_WHIR_CHALLENGE, {r[i]});
      K = h.eval(r[i]);
      whir_sumcheck_step2(arr, b, r[i]);
    }
    vector<F> new_cw;
    vector<vector<_hash>> new_MT;
    Whir_Commit_initial(arr, new_cw, new_MT, 2 * cur_rate, whir_k);
    rec(T_WHIR_ROOT, 1, new_MT.back()[0].arr, 32);
    vector<int> queries;
    vector<F> ys = whir_query(codeword, MT, r, queries, cur_rate);
    {
      vector<uint32_t> q(queries.begin(), queries.end());
      rec(T_WHIR_QUERIES, (uint32_t)q.size(), q.data(), 4);
      vector<F> replies;
      for (int qi : queries)
        for (int j = 0; j < whir_k; j++) replies.push_back(codeword[qi + j * codeword.size() / whir_k]);
      recF(T_WHIR_REPLIES, replies);
      recF(T_WHIR_ANSWERS, ys);
      vector<uint8_t> paths;
      for (int qi : queries) {
        vector<_hash> p = merkle_tree::merkle_tree_prover::open_tree_blake(MT, qi);
        for (auto &h : p) paths.insert(paths.end(), h.arr, h.arr + 32);
      }
      rec(T_WHIR_PATHS, (uint32_t)(paths.size() / 32), paths.data(), 32);
    }
    for (size_t i = 0; i < queries.size(); i++)
      queries[i] = queries[i] * (whir_k * new_cw.size() / codeword.size());
    codeword = new_cw;
    MT = new_MT;
    vector<F> ch = update_betas(b, queries, (int)new_cw.size());
    recF(T_WHIR_COMBINE, ch);
    for (size_t i = 0; i < ch.size(); i++) K += ch[i] * ys[i];
    recF(T_WHIR_K, {K});
    cur_rate *= 2;
    if ((int)arr.size() <= whir_k) break;
  }
  recF(T_FINAL_POLY, arr);
  {
    vector<F> fin_cw;
    vector<vector<_hash>> fin_MT = MT;
    Whir_Commit(arr, fin_cw, fin_MT, cur_rate);
    for (size_t i = 0; i < fin_cw.size(); i++)
      if (fin_cw[i] != codeword[i]) { fprintf(stderr, "verification step 1 failed\n"); return 2; }
    F Kc = K;
    for (size_t i = 0; i < arr.size(); i++) Kc -= arr[i] * b[i];
    if (Kc != F(0)) { fprintf(stderr, "verification step 2 failed\n"); return 2; }
  }
  vector<F> rf;
  for (int i = 0; i < (int)log2(arr.size()); i++) rf.push_back(F::_random());
  recF(T_FINAL_POINT, rf);
  recF(T_FINAL_EVAL, {evaluate_vector(b, rf)});
  long next_after = random();

  if (check) {
    // Unmodified reference: Whir_Open on the same inputs and PRNG start.
    srandom(prng_seed);
    vector<pair<F, vector<F>>> claims = {std::make_pair(v1[0], chal)};
    Whir_Open(w_copy, cw_copy, MT_copy, claims, rate);
    long ref_next = random();
    if (ref_next != next_after) { fprintf(stderr, "PRNG position differs from Whir_Open\n"); return 3; }
    if (w_copy.size() != arr.size()) { fprintf(stderr, "final size differs\n"); return 3; }
    for (size_t i = 0; i < arr.size(); i++)
      if (w_copy[i] != arr[i]) { fprintf(stderr, "final poly differs from Whir_Open\n"); return 3; }
    if (cw_copy.size() != codeword.size()) { fprintf(stderr, "final codeword differs\n"); return 3; }
    for (size_t i = 0; i < codeword.size(); i++)
      if (cw_copy[i] != codeword[i]) { fprintf(stderr, "final codeword differs\n"); return 3; }
    fprintf(stderr, "Whir_Open agrees (verifier checks passed)\n");
  }
  (void)statebuf;
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 2) { fprintf(stderr, "usage: see header\n"); return 1; }
  std::string c = argv[1];
  auto I = [&](int k) { return atoi(argv[k]); };
  auto U = [&](int k) { return (uint64_t)strtoull(argv[k], nullptr, 0); };
  if (c == "field") return cmd_field(I(2), U(3));
  if (c == "blake3") return cmd_blake3(I(2), U(3));
  if (c == "fft") return cmd_fft(I(2), I(3), U(4), false);
  if (c == "pfft") return cmd_fft(I(2), 0, U(3), true);
  if (c == "merkle") return cmd_merkle(I(2), U(3));
  if (c == "fs") return cmd_fs(I(2), U(3));
  if (c == "prng") return cmd_prng(I(2), (unsigned)U(3));
  if (c == "beta") return cmd_beta(I(2), U(3));
  if (c == "tensor") return cmd_tensor(I(2), I(3), I(4), U(5));
  if (c == "betas") return cmd_betas(I(2), I(3), I(4), U(5), (unsigned)U(6));
  if (c == "prove") return cmd_prove(I(2), I(3), U(4), (unsigned)U(5), argc > 6 && atoi(argv[6]));
  fprintf(stderr, "unknown command %s\n", argv[1]);
  return 1;
}
